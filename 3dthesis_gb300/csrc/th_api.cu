// C ABI: context life cycle, node lists, temperature evaluation and snapshots.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/thesis_gb300.h"
#include "th_ctx.h"
#include "th_kernels.h"
#include "th_nodes.cuh"
#include "th_track.h"

static thread_local std::string g_create_error;

th_status th_fail(th_ctx* ctx, th_status code, const std::string& msg) {
  if (ctx) ctx->err = msg; else g_create_error = msg;
  return code;
}

th_status th_cuda_check(th_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return TH_OK;
  return th_fail(ctx, TH_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TH_CUDA(ctx, call)                                        \
  do {                                                            \
    th_status st_ = th_cuda_check((ctx), (call), #call);          \
    if (st_ != TH_OK) return st_;                                 \
  } while (0)

// Device allocations of context creation, numbered from 1 per creation.  The test knob
// THESIS_GB300_FAIL_ALLOC=n makes the n-th one fail as an out-of-memory cudaMalloc would,
// without allocating, so the failure path of creation can be exercised.
static thread_local int g_create_allocs = 0;

static cudaError_t create_malloc(void** p, size_t bytes) {
  ++g_create_allocs;
  if (const char* env = std::getenv("THESIS_GB300_FAIL_ALLOC"))
    if (std::atoi(env) == g_create_allocs) { *p = nullptr; return cudaErrorMemoryAllocation; }
  return cudaMalloc(p, bytes);
}

static th_status alloc_nodes(th_ctx* ctx, int cap) {
  if (ctx->node_mem) cudaFree(ctx->node_mem);
  ctx->node_mem = nullptr;
  const size_t bytes = (size_t)cap * (8 * sizeof(double) + 10 * sizeof(float));
  {
    const th_status st = th_cuda_check(ctx, create_malloc(&ctx->node_mem, bytes), "cudaMalloc");
    if (st != TH_OK) return st;
  }
  double* d = (double*)ctx->node_mem;
  float* f = (float*)(d + 8 * (size_t)cap);
  NodeBufView& nb = ctx->nb;
  nb.cap = cap;
  nb.x = d; nb.y = d + cap; nb.z = d + 2 * (size_t)cap; nb.ipx = d + 3 * (size_t)cap;
  nb.ipy = d + 4 * (size_t)cap; nb.ipz = d + 5 * (size_t)cap; nb.dtau = d + 6 * (size_t)cap; nb.amp = d + 7 * (size_t)cap;
  nb.kx = f; nb.ky = f + cap; nb.kz = f + 2 * (size_t)cap; nb.w = f + 3 * (size_t)cap;
  nb.xh = f + 4 * (size_t)cap; nb.xl = f + 5 * (size_t)cap; nb.yh = f + 6 * (size_t)cap; nb.yl = f + 7 * (size_t)cap;
  nb.zh = f + 8 * (size_t)cap; nb.zl = f + 9 * (size_t)cap;
  return TH_OK;
}

// Reads the error bits and node count left by the last generation; grows the node
// buffer and asks for a retry when it was too small.
static th_status check_nodes(th_ctx* ctx, bool* retry) {
  int h[2];
  TH_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_small, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const int count = h[0], err = h[1];
  *retry = false;
  if (err & thdev::ERR_WALK_LIMIT) return th_fail(ctx, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
  if (err & thdev::ERR_NODE_CAPACITY) {
    const long long need = (long long)count + 1024;
    if (need > (1 << 26)) return th_fail(ctx, TH_ERR_CAPACITY, "node list larger than 2^26 nodes");
    TH_CUDA(ctx, cudaMemsetAsync(ctx->d_small + 1, 0, sizeof(int), ctx->stream));
    th_status st = alloc_nodes(ctx, (int)need);
    if (st != TH_OK) return st;
    *retry = true;
  }
  ctx->last_count = count;
  return TH_OK;
}

th_status th_gen_nodes_checked(th_ctx* ctx, double t, bool is_sol) {
  for (int attempt = 0; attempt < 3; ++attempt) {
    th_launch_nodes(ctx->dp, t, is_sol, ctx->nb, ctx->d_small, ctx->d_small + 1, ctx->stream);
    TH_CUDA(ctx, cudaGetLastError());
    bool retry = false;
    th_status st = check_nodes(ctx, &retry);
    if (st != TH_OK || !retry) return st;
  }
  return th_fail(ctx, TH_ERR_CAPACITY, "node buffer growth did not converge");
}

th_status th_ensure(th_ctx* ctx, void** ptr, size_t* cap_bytes, size_t need) {
  if (*cap_bytes >= need && *ptr) return TH_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  *cap_bytes = 0;
  TH_CUDA(ctx, cudaMalloc(ptr, need));
  *cap_bytes = need;
  return TH_OK;
}

extern "C" {

th_status th_ctx_create_from_deck(const char* param_input, int32_t precision, th_ctx** out) {
  if (!param_input || !out) return th_fail(nullptr, TH_ERR_INVALID, "null argument");
  *out = nullptr;
  if (precision != TH_FP64 && precision != TH_FP32_KAHAN) return th_fail(nullptr, TH_ERR_INVALID, "unknown precision");
  th_ctx* ctx = new th_ctx();
  g_create_allocs = 0;
  std::string err;
  if (!th_load_deck(param_input, ctx->hp, err)) {
    delete ctx;
    return th_fail(nullptr, TH_ERR_INVALID, err);
  }
  ctx->precision = precision;
  if (cudaGetDevice(&ctx->device) != cudaSuccess) {
    delete ctx;
    return th_fail(nullptr, TH_ERR_CUDA, "no CUDA device");
  }
  auto fail = [&](th_status st) {
    g_create_error = ctx->err;
    th_ctx_destroy(ctx);
    return st;
  };
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    ctx->err = "cudaStreamCreate failed";
    return fail(TH_ERR_CUDA);
  }
  cudaEventCreate(&ctx->ev0);
  cudaEventCreate(&ctx->ev1);
  const std::vector<DevSeg> segs = th_pack_segments(ctx->hp);
  if (th_cuda_check(ctx, create_malloc((void**)&ctx->d_segs, segs.size() * sizeof(DevSeg)), "cudaMalloc") != TH_OK)
    return fail(TH_ERR_CUDA);
  if (th_cuda_check(ctx, cudaMemcpy(ctx->d_segs, segs.data(), segs.size() * sizeof(DevSeg), cudaMemcpyHostToDevice),
                    "cudaMemcpy") != TH_OK)
    return fail(TH_ERR_CUDA);
  th_make_dev_problem(ctx->hp, ctx->d_segs, ctx->dp);
  if (ctx->hp.custom) {                     // the custom points' coordinates, read by point_xyz
    const size_t n = (size_t)ctx->hp.pnum;
    if (th_cuda_check(ctx, create_malloc((void**)&ctx->d_custom, 3 * n * sizeof(double)), "cudaMalloc") != TH_OK)
      return fail(TH_ERR_CUDA);
    const std::vector<double>* c[3] = {&ctx->hp.px, &ctx->hp.py, &ctx->hp.pz};
    for (int a = 0; a < 3; ++a)
      if (th_cuda_check(ctx, cudaMemcpy(ctx->d_custom + a * n, c[a]->data(), n * sizeof(double), cudaMemcpyHostToDevice),
                        "cudaMemcpy") != TH_OK)
        return fail(TH_ERR_CUDA);
    ctx->dp.cx = ctx->d_custom; ctx->dp.cy = ctx->d_custom + n; ctx->dp.cz = ctx->d_custom + 2 * n;
  }
  if (ctx->dp.n_images > TH_MAX_IMAGES) {
    ctx->err = "more boundary images than TH_MAX_IMAGES";
    return fail(TH_ERR_CAPACITY);
  }
  if (th_cuda_check(ctx, create_malloc((void**)&ctx->d_small, 16 * sizeof(int)), "cudaMalloc") != TH_OK)
    return fail(TH_ERR_CUDA);
  if (th_cuda_check(ctx, cudaMemset(ctx->d_small, 0, 16 * sizeof(int)), "cudaMemset") != TH_OK) return fail(TH_ERR_CUDA);
  if (th_cuda_check(ctx, create_malloc((void**)&ctx->d_pairs, 2 * sizeof(unsigned long long)), "cudaMalloc") != TH_OK)
    return fail(TH_ERR_CUDA);
  if (th_cuda_check(ctx, cudaMemset(ctx->d_pairs, 0, 2 * sizeof(unsigned long long)), "cudaMemset") != TH_OK) return fail(TH_ERR_CUDA);
  // capacity: 64 nodes per segment per beam and a margin, times the image count; grown on demand
  size_t segs_total = segs.size();
  int cap = (int)std::min<size_t>((size_t)(64 * segs_total + 4096) * (size_t)ctx->dp.n_images, 1 << 24);
  if (alloc_nodes(ctx, cap) != TH_OK) return fail(TH_ERR_CUDA);
  ctx->shape = TileShape{4, 2};
  *out = ctx;
  return TH_OK;
}

void th_ctx_destroy(th_ctx* ctx) {
  if (!ctx) return;
  int cur = -1;
  cudaGetDevice(&cur);
  if (ctx->device >= 0) cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  th_release_run_state(ctx);
  cudaFree(ctx->node_mem);
  cudaFree(ctx->d_segs);
  cudaFree(ctx->d_custom);
  cudaFree(ctx->d_small);
  cudaFree(ctx->d_pairs);
  cudaFree(ctx->d_T);
  cudaFree(ctx->d_pts);
  cudaFree(ctx->d_Tlist);
  cudaFree(ctx->d_export);
  cudaFree(ctx->multi_mem);
  cudaFree(ctx->d_multi_t);
  cudaFree(ctx->d_multi_count);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (cur >= 0) cudaSetDevice(cur);
  delete ctx;
}

const char* th_last_error(const th_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

static void fill_info(const HostProblem& hp, int precision, th_info* out) {
  std::memset(out, 0, sizeof(*out));
  out->nx = hp.nx; out->ny = hp.ny; out->nz = hp.nz; out->pnum = hp.pnum;
  out->n_beams = (int32_t)hp.beams.size();
  out->n_snapshots = (int32_t)hp.snaps.size();
  out->mode = hp.mode; out->tracking = hp.tracking;
  out->dt = hp.dt; out->end_time = hp.end_time; out->T0 = hp.T0; out->TL = hp.TL;
  out->xmin = hp.xmin; out->xmax = hp.xmax; out->ymin = hp.ymin; out->ymax = hp.ymax; out->zmin = hp.zmin; out->zmax = hp.zmax;
  out->precision = precision;
  int f = 0;
  if (hp.o_T) f |= TH_OUT_T;
  if (hp.o_tSol) f |= TH_OUT_TSOL;
  if (hp.o_G) f |= TH_OUT_G;
  if (hp.o_Gx) f |= TH_OUT_GX;
  if (hp.o_Gy) f |= TH_OUT_GY;
  if (hp.o_Gz) f |= TH_OUT_GZ;
  if (hp.o_V) f |= TH_OUT_V;
  if (hp.o_dTdt) f |= TH_OUT_DTDT;
  if (hp.o_eqFrac) f |= TH_OUT_EQFRAC;
  if (hp.o_depth) f |= TH_OUT_DEPTH;
  if (hp.o_numMelt) f |= TH_OUT_NUMMELT;
  out->out_flags = f;
}

th_status th_get_info(th_ctx* ctx, th_info* out) {
  if (!ctx || !out) return th_fail(ctx, TH_ERR_INVALID, "null argument");
  fill_info(ctx->hp, ctx->precision, out);
  return TH_OK;
}

th_status th_deck_info(const char* param_input, th_info* out) {
  if (!param_input || !out) {
    g_create_error = "null argument";
    return TH_ERR_INVALID;
  }
  HostProblem hp;
  std::string err;
  if (!th_load_deck(param_input, hp, err)) {
    g_create_error = err;
    return TH_ERR_INVALID;
  }
  fill_info(hp, -1, out);
  return TH_OK;
}

double th_snapshot_time(th_ctx* ctx, int32_t idx) {
  if (!ctx || idx < 0 || idx >= (int32_t)ctx->hp.snaps.size()) return NAN;
  return ctx->hp.snaps[idx];
}

th_status th_nodes(th_ctx* ctx, double t, int32_t is_sol, double* out, int32_t cap, int32_t* n_out) {
  if (!ctx || (!out && cap > 0) || cap < 0) return th_fail(ctx, TH_ERR_INVALID, "bad argument");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  th_status st = th_gen_nodes_checked(ctx, t, is_sol != 0);
  if (st != TH_OK) return st;
  const int n = ctx->last_count;
  if (n_out) *n_out = n;
  const int m = std::min(n, (int)cap);
  if (m > 0) {
    const int dcap = ctx->nb.cap;
    st = th_ensure(ctx, (void**)&ctx->d_export, &ctx->export_bytes, (size_t)8 * dcap * sizeof(double));
    if (st != TH_OK) return st;
    th_launch_nodes_export(ctx->nb, ctx->d_small, ctx->d_export, dcap, ctx->stream);
    TH_CUDA(ctx, cudaGetLastError());
    for (int c = 0; c < 8; ++c)
      TH_CUDA(ctx, cudaMemcpyAsync(out + (size_t)c * cap, ctx->d_export + (size_t)c * dcap, m * sizeof(double),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    TH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return TH_OK;
}

th_status th_calc_T(th_ctx* ctx, double t, const int64_t* pts, int64_t n, double* T_out) {
  if (!ctx || !T_out || n < 0) return th_fail(ctx, TH_ERR_INVALID, "bad argument");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  if (!pts) {
    if (n != ctx->hp.pnum) return th_fail(ctx, TH_ERR_INVALID, "pts == NULL needs n == pnum");
    th_status st = th_gen_nodes_checked(ctx, t, false);
    if (st != TH_OK) return st;
    st = th_ensure(ctx, (void**)&ctx->d_T, &ctx->T_bytes, (size_t)ctx->hp.pnum * sizeof(double));
    if (st != TH_OK) return st;
    th_launch_grid_sum(ctx->dp, ctx->nb, ctx->d_small, ctx->d_T, ctx->precision, ctx->shape, ctx->d_pairs, ctx->stream);
    TH_CUDA(ctx, cudaGetLastError());
    TH_CUDA(ctx, cudaMemcpyAsync(T_out, ctx->d_T, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    TH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return TH_OK;
  }
  for (int64_t i = 0; i < n; ++i)
    if (pts[i] < 0 || pts[i] >= ctx->hp.pnum) return th_fail(ctx, TH_ERR_INVALID, "point id out of range");
  th_status st = th_gen_nodes_checked(ctx, t, false);
  if (st != TH_OK) return st;
  st = th_ensure(ctx, (void**)&ctx->d_pts, &ctx->pts_bytes, std::max<int64_t>(n, 1) * sizeof(int64_t));
  if (st != TH_OK) return st;
  st = th_ensure(ctx, (void**)&ctx->d_Tlist, &ctx->Tlist_bytes, std::max<int64_t>(n, 1) * sizeof(double));
  if (st != TH_OK) return st;
  if (n == 0) return TH_OK;
  TH_CUDA(ctx, cudaMemcpyAsync(ctx->d_pts, pts, n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  th_launch_list_sum(ctx->dp, ctx->nb, ctx->d_small, ctx->d_pts, n, ctx->d_Tlist, ctx->precision, ctx->d_pairs,
                     ctx->stream);
  TH_CUDA(ctx, cudaGetLastError());
  TH_CUDA(ctx, cudaMemcpyAsync(T_out, ctx->d_Tlist, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  TH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TH_OK;
}

th_status th_calc_T_device(th_ctx* ctx, double t, const int64_t* d_pts, int64_t n, double* d_T, void* stream) {
  if (!ctx || !d_T || n < 0) return th_fail(ctx, TH_ERR_INVALID, "bad argument");
  if (!d_pts && n != ctx->hp.pnum) return th_fail(ctx, TH_ERR_INVALID, "d_pts == NULL needs n == pnum");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  // No host synchronisation here: device-side errors (node capacity, walk limit) stay
  // latched in the context and are reported by th_sync or the next synchronous call.
  th_launch_nodes(ctx->dp, t, false, ctx->nb, ctx->d_small, ctx->d_small + 1, s);
  if (d_pts) th_launch_list_sum(ctx->dp, ctx->nb, ctx->d_small, d_pts, n, d_T, ctx->precision, ctx->d_pairs, s);
  else th_launch_grid_sum(ctx->dp, ctx->nb, ctx->d_small, d_T, ctx->precision, ctx->shape, ctx->d_pairs, s);
  TH_CUDA(ctx, cudaGetLastError());
  return TH_OK;
}

// Node lists of ntimes times in one launch (a block per time, as Integrate_Parallel
// precomputes several future lists, src/Calc.cpp:21-46), then each time's sum into
// d_T + i * n.  Enqueued on the stream without host synchronisation; node-list errors are
// latched for th_sync.
th_status th_calc_T_times_device(th_ctx* ctx, const double* times, int32_t ntimes, const int64_t* d_pts, int64_t n,
                                 double* d_T, void* stream) {
  if (!ctx || !times || ntimes <= 0 || !d_T || n < 0) return th_fail(ctx, TH_ERR_INVALID, "bad argument");
  if (!d_pts && n != ctx->hp.pnum) return th_fail(ctx, TH_ERR_INVALID, "d_pts == NULL needs n == pnum");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  if (ctx->multi_slots < ntimes || ctx->multi_cap != ctx->nb.cap) {
    TH_CUDA(ctx, cudaStreamSynchronize(s));          // the old buffers may still be read
    cudaFree(ctx->multi_mem); cudaFree(ctx->d_multi_t); cudaFree(ctx->d_multi_count);
    ctx->multi_mem = nullptr; ctx->d_multi_t = nullptr; ctx->d_multi_count = nullptr;
    const int slots = std::max(ntimes, ctx->multi_slots), cap = ctx->nb.cap;
    TH_CUDA(ctx, cudaMalloc(&ctx->multi_mem, (size_t)slots * cap * (8 * sizeof(double) + 10 * sizeof(float))));
    TH_CUDA(ctx, cudaMalloc(&ctx->d_multi_t, slots * sizeof(double)));
    TH_CUDA(ctx, cudaMalloc(&ctx->d_multi_count, slots * sizeof(int)));
    ctx->multi_slots = slots;
    ctx->multi_cap = cap;
  }
  const size_t cap = (size_t)ctx->multi_slots * ctx->multi_cap;
  double* d = (double*)ctx->multi_mem;
  float* f = (float*)(d + 8 * cap);
  NodeWindow w{};
  NodeBufView& nb = w.nb;
  nb.cap = (int)cap;
  nb.x = d; nb.y = d + cap; nb.z = d + 2 * cap; nb.ipx = d + 3 * cap; nb.ipy = d + 4 * cap; nb.ipz = d + 5 * cap;
  nb.dtau = d + 6 * cap; nb.amp = d + 7 * cap;
  nb.kx = f; nb.ky = f + cap; nb.kz = f + 2 * cap; nb.w = f + 3 * cap; nb.xh = f + 4 * cap; nb.xl = f + 5 * cap;
  nb.yh = f + 6 * cap; nb.yl = f + 7 * cap; nb.zh = f + 8 * cap; nb.zl = f + 9 * cap;
  w.slot_cap = ctx->multi_cap;
  w.nslots = ctx->multi_slots;
  w.count = ctx->d_multi_count;
  w.t = ctx->d_multi_t;
  // from pageable memory the copy is staged before the call returns; in stream order it
  // lands after the previous call's kernels have read the times
  TH_CUDA(ctx, cudaMemcpyAsync(ctx->d_multi_t, times, ntimes * sizeof(double), cudaMemcpyHostToDevice, s));
  th_launch_nodes_window(ctx->dp, w, 0, ntimes, false, ctx->d_small + 1, s);
  for (int i = 0; i < ntimes; ++i) {
    NodeBufView v = nb;
    const size_t off = (size_t)i * ctx->multi_cap;
    v.x += off; v.y += off; v.z += off; v.ipx += off; v.ipy += off; v.ipz += off; v.dtau += off; v.amp += off;
    v.kx += off; v.ky += off; v.kz += off; v.w += off; v.xh += off; v.xl += off; v.yh += off; v.yl += off;
    v.zh += off; v.zl += off;
    v.cap = ctx->multi_cap;
    double* out = d_T + (size_t)i * n;
    if (d_pts) th_launch_list_sum(ctx->dp, v, ctx->d_multi_count + i, d_pts, n, out, ctx->precision, ctx->d_pairs, s);
    else th_launch_grid_sum(ctx->dp, v, ctx->d_multi_count + i, out, ctx->precision, ctx->shape, ctx->d_pairs, s);
  }
  TH_CUDA(ctx, cudaGetLastError());
  return TH_OK;
}

th_status th_sync(th_ctx* ctx, void* stream) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  if (stream) TH_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
  int h[2];
  TH_CUDA(ctx, cudaMemcpyAsync(h, ctx->d_small, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (h[1] & thdev::ERR_WALK_LIMIT) return th_fail(ctx, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
  if (h[1] & thdev::ERR_NODE_CAPACITY) {
    // grow for the next call; results enqueued since the overflow are incomplete
    TH_CUDA(ctx, cudaMemsetAsync(ctx->d_small + 1, 0, sizeof(int), ctx->stream));
    th_status st = alloc_nodes(ctx, h[0] + 1024);
    if (st != TH_OK) return st;
    return th_fail(ctx, TH_ERR_CAPACITY, "a node list outgrew its buffer; the buffer has grown, repeat the calls");
  }
  return TH_OK;
}

th_status th_snapshot(th_ctx* ctx, int32_t idx, double* T_out) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  if (ctx->hp.mode != 0 || idx < 0 || idx >= (int32_t)ctx->hp.snaps.size())
    return th_fail(ctx, TH_ERR_INVALID, "no such snapshot");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  th_status st = th_gen_nodes_checked(ctx, ctx->hp.snaps[idx], false);
  if (st != TH_OK) return st;
  st = th_ensure(ctx, (void**)&ctx->d_T, &ctx->T_bytes, (size_t)ctx->hp.pnum * sizeof(double));
  if (st != TH_OK) return st;
  TH_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  th_launch_grid_sum(ctx->dp, ctx->nb, ctx->d_small, ctx->d_T, ctx->precision, ctx->shape, ctx->d_pairs, ctx->stream);
  TH_CUDA(ctx, cudaGetLastError());
  TH_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  if (T_out)
    TH_CUDA(ctx, cudaMemcpyAsync(T_out, ctx->d_T, ctx->hp.pnum * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  TH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  cudaEventElapsedTime(&ctx->last_ms, ctx->ev0, ctx->ev1);
  ctx->T_valid = true;
  return TH_OK;
}

th_status th_pairs(th_ctx* ctx, int64_t* out) {
  if (!ctx || !out) return th_fail(ctx, TH_ERR_INVALID, "null argument");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  unsigned long long v = 0;
  TH_CUDA(ctx, cudaMemcpyAsync(&v, ctx->d_pairs, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
  TH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *out = (int64_t)v;
  return TH_OK;
}

th_status th_last_kernel_ms(th_ctx* ctx, float* out) {
  if (!ctx || !out) return th_fail(ctx, TH_ERR_INVALID, "null argument");
  *out = ctx->last_ms;
  return TH_OK;
}

// Times the whole-grid kernel of snapshot idx with every supported tile shape (the node
// list is generated once; four launches per shape, the first dropped, the best kept) and
// keeps the fastest shape for the context.
th_status th_autotune(th_ctx* ctx, int32_t idx, int32_t* kp_out, int32_t* kch_out) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  if (ctx->hp.mode != 0 || idx < 0 || idx >= (int32_t)ctx->hp.snaps.size())
    return th_fail(ctx, TH_ERR_INVALID, "no such snapshot");
  TH_CUDA(ctx, cudaSetDevice(ctx->device));
  th_status st = th_gen_nodes_checked(ctx, ctx->hp.snaps[idx], false);
  if (st != TH_OK) return st;
  st = th_ensure(ctx, (void**)&ctx->d_T, &ctx->T_bytes, (size_t)ctx->hp.pnum * sizeof(double));
  if (st != TH_OK) return st;
  const TileShape shapes[7] = {{4, 2}, {4, 1}, {4, 4}, {2, 2}, {2, 4}, {8, 1}, {8, 2}};
  float best = 1e30f;
  TileShape best_shape = ctx->shape;
  for (const TileShape& sh : shapes) {
    float t_best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
      TH_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
      th_launch_grid_sum(ctx->dp, ctx->nb, ctx->d_small, ctx->d_T, ctx->precision, sh, ctx->d_pairs, ctx->stream);
      TH_CUDA(ctx, cudaGetLastError());
      TH_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
      TH_CUDA(ctx, cudaEventSynchronize(ctx->ev1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
      if (rep > 0) t_best = std::min(t_best, ms);
    }
    if (t_best < best) { best = t_best; best_shape = sh; }
  }
  ctx->shape = best_shape;
  ctx->T_valid = false;
  if (kp_out) *kp_out = best_shape.kp;
  if (kch_out) *kch_out = best_shape.kch;
  return TH_OK;
}

// Tile shape of the whole-grid kernels (k-points per thread, k-chunks per tile).
th_status th_set_tile_shape(th_ctx* ctx, int32_t kp, int32_t kch) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  TileShape sh{kp, kch};
  if (!th_tile_shape_supported(sh)) return th_fail(ctx, TH_ERR_INVALID, "unsupported tile shape");
  ctx->shape = sh;
  return TH_OK;
}

}  // extern "C"
