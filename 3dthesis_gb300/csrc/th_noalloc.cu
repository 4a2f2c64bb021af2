// Allocation-free temperature evaluation (th_calc_T_noalloc).
//
// Who needs it: callers that hand this library their own device buffers and may not
// allocate device memory themselves or let the library do it - a host code whose device
// memory is owned by its own pool or fixed budget after start-up, or a solver that calls
// this from its time loop, where cudaMalloc / cudaFree would synchronise the device and
// could fail under memory pressure.  The other evaluation calls keep their node list in
// the context's buffer, which th_sync and the synchronous calls enlarge (cudaFree +
// cudaMalloc) when a list outgrows it.  This call never allocates: its node list lives
// in the fixed array below, and a list that does not fit is an error.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "th_ctx.h"
#include "th_kernels.h"
#include "th_nodes.cuh"

namespace {

// Largest node list the static scratch holds.  Every GPU that loads the library keeps
// this array (kStaticBytes, about 1.7 MB) until the process exits.
constexpr int kStaticNodes = 16384;
constexpr size_t kHeader = 256;   // [0] node count, [1] error bits
constexpr size_t kStaticBytes = kHeader + (size_t)kStaticNodes * (8 * sizeof(double) + 10 * sizeof(float));

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `device` (current).  Host code cannot use the
// array's name as an address: that is a host-side stand-in.  Looked up once per device.
th_status scratch_address(th_ctx* ctx, int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return th_fail(ctx, TH_ERR_CAPACITY, "device ordinal above 63");
  std::lock_guard<std::mutex> g(g_lock);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return th_cuda_check(ctx, e, "cudaGetSymbolAddress");
    g_scratch_addr[device] = p;
  }
  *out = (unsigned char*)g_scratch_addr[device];
  return TH_OK;
}

NodeBufView static_view(unsigned char* base) {
  NodeBufView nb;
  const size_t cap = kStaticNodes;
  double* d = (double*)(base + kHeader);
  float* f = (float*)(d + 8 * cap);
  nb.cap = kStaticNodes;
  nb.x = d; nb.y = d + cap; nb.z = d + 2 * cap; nb.ipx = d + 3 * cap;
  nb.ipy = d + 4 * cap; nb.ipz = d + 5 * cap; nb.dtau = d + 6 * cap; nb.amp = d + 7 * cap;
  nb.kx = f; nb.ky = f + cap; nb.kz = f + 2 * cap; nb.w = f + 3 * cap;
  nb.xh = f + 4 * cap; nb.xl = f + 5 * cap; nb.yh = f + 6 * cap; nb.yl = f + 7 * cap;
  nb.zh = f + 8 * cap; nb.zl = f + 9 * cap;
  return nb;
}

}  // namespace

extern "C" th_status th_calc_T_noalloc(th_ctx* ctx, double t, const int64_t* d_pts, int64_t n, double* d_T,
                                       void* stream) {
  if (!ctx || !d_T || n < 0) return th_fail(ctx, TH_ERR_INVALID, "bad argument");
  if (!d_pts && n != ctx->hp.pnum) return th_fail(ctx, TH_ERR_INVALID, "d_pts == NULL needs n == pnum");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return th_cuda_check(ctx, e, "cudaSetDevice");
  unsigned char* base = nullptr;
  th_status st = scratch_address(ctx, ctx->device, &base);
  if (st != TH_OK) return st;
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  int* hdr = (int*)base;
  const NodeBufView nb = static_view(base);
  // the array keeps the previous call's contents: the count and error bits start at zero
  e = cudaMemsetAsync(hdr, 0, 2 * sizeof(int), s);
  if (e != cudaSuccess) return th_cuda_check(ctx, e, "cudaMemsetAsync");
  th_launch_nodes(ctx->dp, t, false, nb, hdr, hdr + 1, s);
  if (d_pts) th_launch_list_sum(ctx->dp, nb, hdr, d_pts, n, d_T, ctx->precision, ctx->d_pairs, s);
  else th_launch_grid_sum(ctx->dp, nb, hdr, d_T, ctx->precision, ctx->shape, ctx->d_pairs, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return th_cuda_check(ctx, e, "kernel launch");
  int h[2] = {0, 0};
  e = cudaMemcpyAsync(h, hdr, sizeof(h), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return th_cuda_check(ctx, e, "cudaMemcpyAsync");
  if (h[1] & thdev::ERR_WALK_LIMIT) return th_fail(ctx, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
  if (h[1] & thdev::ERR_NODE_CAPACITY)
    return th_fail(ctx, TH_ERR_CAPACITY,
                   "node list of " + std::to_string(h[0]) + " nodes exceeds the static maximum of " +
                       std::to_string(kStaticNodes) + " nodes of th_calc_T_noalloc; d_T is not valid");
  return TH_OK;
}
