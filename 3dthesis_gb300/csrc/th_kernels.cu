// Node generation and point x node temperature kernels for sm_103a.
//
// The temperature at a point is T0 + sum_n dtau_n amp_n exp(-3 sum_d (p_d - x_nd)^2 / phi_nd)
// (the reference's Grid::Calc_T, src/Grid.cpp:275-314).  The sum is bound by FP32-pipe and
// MUFU issue, not by memory: every node is read once per CTA from shared memory as a
// warp-wide broadcast, every point is owned by one thread for the whole node loop, and
// each point's result is written once.
#include <cstdint>
#include <cuda_runtime.h>

#include "th_kernels.h"
#include "th_device.cuh"

namespace {

using namespace thdev;

__global__ void __launch_bounds__(kGenThreads) k_nodes_block(DevProblem P, double t, int is_sol, NodeBufView nb,
                                                             int* count, int* err) {
  __shared__ GenShared sh;
  gen_list_block(P, t, is_sol != 0, nb, count, err, sh);
}

// ---------------------------------------------------------------- whole-grid sums
constexpr int kThreads = 256;
constexpr int kChunk = 256;   // nodes staged in shared memory per pass
constexpr int kCJ = 8;        // tile width along j

// FP32 + Kahan.  Offsets from the tile centre are formed in FP64 and rounded once, so the
// FP32 differences keep ~1e-7 relative accuracy on the tile's scale; the exponent is
// evaluated as exp2 with -3 log2(e) folded into the per-node coefficients.
template <int KP, int KCH>
__global__ void __launch_bounds__(kThreads) k_grid_fp32(DevProblem P, NodeBufView nb, const int* count,
                                                        double* __restrict__ T, int ntj, int ntk,
                                                        unsigned long long* pairs) {
  constexpr int CI = kThreads / KCH / kCJ, TK = KP * KCH;
  __shared__ float4 sA[kChunk], sB[kChunk];
  const int nn = min(*count, nb.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(pairs, (unsigned long long)nn * (unsigned long long)P.pnum);
  const int tile = blockIdx.x;
  const int tk = tile % ntk, tij = tile / ntk, tj = tij % ntj, ti = tij / ntj;
  const int kc = threadIdx.x % KCH, col = threadIdx.x / KCH, ci = col / kCJ, cj = col % kCJ;
  const double Xo = coord(P.gx, P.xmin, P.xmax, P.hx, ti * CI + CI / 2);
  const double Yo = coord(P.gy, P.ymin, P.ymax, P.hy, tj * kCJ + kCJ / 2);
  const double Zo = coord(P.gz, P.zmin, P.zmax, P.hz, tk * TK + TK / 2);
  const int i = ti * CI + ci, j = tj * kCJ + cj, k0 = tk * TK + kc * KP;
  const float px = __double2float_rn(coord(P.gx, P.xmin, P.xmax, P.hx, i) - Xo);
  const float py = __double2float_rn(coord(P.gy, P.ymin, P.ymax, P.hy, j) - Yo);
  float pz[KP], s[KP], c[KP];
#pragma unroll
  for (int q = 0; q < KP; ++q) {
    pz[q] = __double2float_rn(coord(P.gz, P.zmin, P.zmax, P.hz, k0 + q) - Zo);
    s[q] = 0.f; c[q] = 0.f;
  }
  for (int base = 0; base < nn; base += kChunk) {
    __syncthreads();
    const int idx = base + threadIdx.x;
    if (idx < nn) {
      sA[threadIdx.x] = make_float4(__double2float_rn(nb.x[idx] - Xo), __double2float_rn(nb.y[idx] - Yo),
                                    __double2float_rn(nb.z[idx] - Zo), nb.kx[idx]);
      sB[threadIdx.x] = make_float4(nb.ky[idx], nb.kz[idx], nb.w[idx], 0.f);
    }
    __syncthreads();
    const int m = min(kChunk, nn - base);
#pragma unroll 2
    for (int n = 0; n < m; ++n) {
      const float4 a = sA[n], b = sB[n];
      const float dx = px - a.x, dy = py - a.y;
      const float exy = fmaf(dy * dy, b.x, dx * dx * a.w);
#pragma unroll
      for (int q = 0; q < KP; ++q) {
        const float dz = pz[q] - a.z;
        const float v = ex2_approx(fmaf(dz * dz, b.y, exy)) * b.z;
        const float y = v - c[q];
        const float t = s[q] + y;
        c[q] = (t - s[q]) - y;
        s[q] = t;
      }
    }
  }
  if (i < P.nx && j < P.ny) {
    const int64_t row = ((int64_t)i * P.ny + j) * P.nz;
#pragma unroll
    for (int q = 0; q < KP; ++q)
      if (k0 + q < P.nz) T[row + k0 + q] = P.T0 + ((double)s[q] - (double)c[q]);
  }
}

// Plain FP64 (the reference's arithmetic, one libdevice exp per pair).
template <int KP, int KCH>
__global__ void __launch_bounds__(kThreads) k_grid_fp64(DevProblem P, NodeBufView nb, const int* count,
                                                        double* __restrict__ T, int ntj, int ntk,
                                                        unsigned long long* pairs) {
  constexpr int CI = kThreads / KCH / kCJ, TK = KP * KCH;
  __shared__ double2 sN[kChunk][4];
  const int nn = min(*count, nb.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(pairs, (unsigned long long)nn * (unsigned long long)P.pnum);
  const int tile = blockIdx.x;
  const int tk = tile % ntk, tij = tile / ntk, tj = tij % ntj, ti = tij / ntj;
  const int kc = threadIdx.x % KCH, col = threadIdx.x / KCH, ci = col / kCJ, cj = col % kCJ;
  const int i = ti * CI + ci, j = tj * kCJ + cj, k0 = tk * TK + kc * KP;
  const double xp = coord(P.gx, P.xmin, P.xmax, P.hx, i);
  const double yp = coord(P.gy, P.ymin, P.ymax, P.hy, j);
  double zp[KP], s[KP];
#pragma unroll
  for (int q = 0; q < KP; ++q) { zp[q] = coord(P.gz, P.zmin, P.zmax, P.hz, k0 + q); s[q] = 0.0; }
  for (int base = 0; base < nn; base += kChunk) {
    __syncthreads();
    const int idx = base + threadIdx.x;
    if (idx < nn) {
      sN[threadIdx.x][0] = make_double2(nb.x[idx], nb.y[idx]);
      sN[threadIdx.x][1] = make_double2(nb.z[idx], nb.ipx[idx]);
      sN[threadIdx.x][2] = make_double2(nb.ipy[idx], nb.ipz[idx]);
      sN[threadIdx.x][3] = make_double2(nb.dtau[idx] * nb.amp[idx], 0.0);
    }
    __syncthreads();
    const int m = min(kChunk, nn - base);
    for (int n = 0; n < m; ++n) {
      const double2 a = sN[n][0], b = sN[n][1], c2 = sN[n][2], d = sN[n][3];
      const double dx = xp - a.x, dy = yp - a.y;
      const double exy = dx * dx * b.y + dy * dy * c2.x;
#pragma unroll
      for (int q = 0; q < KP; ++q) {
        const double dz = zp[q] - b.x;
        s[q] += d.x * exp(-3.0 * (exy + dz * dz * c2.y));
      }
    }
  }
  if (i < P.nx && j < P.ny) {
    const int64_t row = ((int64_t)i * P.ny + j) * P.nz;
#pragma unroll
    for (int q = 0; q < KP; ++q)
      if (k0 + q < P.nz) T[row + k0 + q] = P.T0 + s[q];
  }
}

// ---------------------------------------------------------------- listed points
// FP32 + Kahan for arbitrary points.  Point and node coordinates are each split into
// two floats; (ph - nh) + (pl - nl) keeps the difference accurate to ~1e-7 of itself
// wherever the points lie.
__global__ void __launch_bounds__(kThreads) k_list_fp32(DevProblem P, NodeBufView nb, const int* count,
                                                        const int64_t* __restrict__ pts, int64_t n,
                                                        double* __restrict__ T, unsigned long long* pairs) {
  __shared__ float4 sA[kChunk], sB[kChunk], sC[kChunk];
  const int nn = min(*count, nb.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(pairs, (unsigned long long)nn * (unsigned long long)n);
  const int64_t gi = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool live = gi < n;
  double x = 0, y = 0, z = 0;
  if (live) point_xyz(P, pts[gi], x, y, z);
  const float xh = __double2float_rn(x), yh = __double2float_rn(y), zh = __double2float_rn(z);
  const float xl = __double2float_rn(x - (double)xh), yl = __double2float_rn(y - (double)yh),
              zl = __double2float_rn(z - (double)zh);
  float s = 0.f, c = 0.f;
  for (int base = 0; base < nn; base += kChunk) {
    __syncthreads();
    const int idx = base + threadIdx.x;
    if (idx < nn) {
      sA[threadIdx.x] = make_float4(nb.xh[idx], nb.xl[idx], nb.yh[idx], nb.yl[idx]);
      sB[threadIdx.x] = make_float4(nb.zh[idx], nb.zl[idx], nb.kx[idx], nb.ky[idx]);
      sC[threadIdx.x] = make_float4(nb.kz[idx], nb.w[idx], 0.f, 0.f);
    }
    __syncthreads();
    const int m = min(kChunk, nn - base);
    for (int k = 0; k < m; ++k) {
      const float4 a = sA[k], b = sB[k], cc = sC[k];
      const float dx = (xh - a.x) + (xl - a.y);
      const float dy = (yh - a.z) + (yl - a.w);
      const float dz = (zh - b.x) + (zl - b.y);
      const float e = fmaf(dz * dz, cc.x, fmaf(dy * dy, b.w, dx * dx * b.z));
      const float v = ex2_approx(e) * cc.y;
      const float yy = v - c;
      const float t = s + yy;
      c = (t - s) - yy;
      s = t;
    }
  }
  if (live) T[gi] = P.T0 + ((double)s - (double)c);
}

__global__ void __launch_bounds__(kThreads) k_list_fp64(DevProblem P, NodeBufView nb, const int* count,
                                                        const int64_t* __restrict__ pts, int64_t n,
                                                        double* __restrict__ T, unsigned long long* pairs) {
  __shared__ double2 sN[kChunk][4];
  const int nn = min(*count, nb.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(pairs, (unsigned long long)nn * (unsigned long long)n);
  const int64_t gi = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  const bool live = gi < n;
  double x = 0, y = 0, z = 0;
  if (live) point_xyz(P, pts[gi], x, y, z);
  double s = 0.0;
  for (int base = 0; base < nn; base += kChunk) {
    __syncthreads();
    const int idx = base + threadIdx.x;
    if (idx < nn) {
      sN[threadIdx.x][0] = make_double2(nb.x[idx], nb.y[idx]);
      sN[threadIdx.x][1] = make_double2(nb.z[idx], nb.ipx[idx]);
      sN[threadIdx.x][2] = make_double2(nb.ipy[idx], nb.ipz[idx]);
      sN[threadIdx.x][3] = make_double2(nb.dtau[idx] * nb.amp[idx], 0.0);
    }
    __syncthreads();
    const int m = min(kChunk, nn - base);
    for (int k = 0; k < m; ++k) {
      const double2 a = sN[k][0], b = sN[k][1], c2 = sN[k][2], d = sN[k][3];
      const double dx = x - a.x, dy = y - a.y, dz = z - b.x;
      s += d.x * exp(-3.0 * (dx * dx * b.y + dy * dy * c2.x + dz * dz * c2.y));
    }
  }
  if (live) T[gi] = P.T0 + s;
}

__global__ void k_nodes_export(NodeBufView nb, const int* count, double* out, int cap) {
  const int nn = min(*count, min(nb.cap, cap));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
    out[0 * (size_t)cap + i] = nb.x[i];
    out[1 * (size_t)cap + i] = nb.y[i];
    out[2 * (size_t)cap + i] = nb.z[i];
    out[3 * (size_t)cap + i] = nb.ipx[i];
    out[4 * (size_t)cap + i] = nb.ipy[i];
    out[5 * (size_t)cap + i] = nb.ipz[i];
    out[6 * (size_t)cap + i] = nb.dtau[i];
    out[7 * (size_t)cap + i] = log(nb.amp[i]);
  }
}

template <int KP, int KCH>
void launch_grid(const DevProblem& P, const NodeBufView& nb, const int* d_count, double* d_T, int precision,
                 unsigned long long* pairs, cudaStream_t s) {
  constexpr int CI = kThreads / KCH / kCJ, TK = KP * KCH;
  const int nti = (P.nx + CI - 1) / CI, ntj = (P.ny + kCJ - 1) / kCJ, ntk = (P.nz + TK - 1) / TK;
  const int blocks = nti * ntj * ntk;
  if (precision == 0) k_grid_fp64<KP, KCH><<<blocks, kThreads, 0, s>>>(P, nb, d_count, d_T, ntj, ntk, pairs);
  else k_grid_fp32<KP, KCH><<<blocks, kThreads, 0, s>>>(P, nb, d_count, d_T, ntj, ntk, pairs);
}

}  // namespace

void th_launch_nodes(const DevProblem& P, double t, bool is_sol, const NodeBufView& nb, int* d_count, int* d_err,
                     cudaStream_t s) {
  k_nodes_block<<<1, kGenThreads, 0, s>>>(P, t, is_sol ? 1 : 0, nb, d_count, d_err);
}

bool th_tile_shape_supported(TileShape sh) {
  return (sh.kp == 4 && (sh.kch == 1 || sh.kch == 2 || sh.kch == 4)) || (sh.kp == 2 && (sh.kch == 2 || sh.kch == 4)) ||
         (sh.kp == 8 && (sh.kch == 1 || sh.kch == 2));
}

void th_launch_grid_sum(const DevProblem& P, const NodeBufView& nb, const int* d_count, double* d_T, int precision,
                        TileShape sh, unsigned long long* pairs, cudaStream_t s) {
  if (sh.kp == 4 && sh.kch == 1) launch_grid<4, 1>(P, nb, d_count, d_T, precision, pairs, s);
  else if (sh.kp == 4 && sh.kch == 4) launch_grid<4, 4>(P, nb, d_count, d_T, precision, pairs, s);
  else if (sh.kp == 2 && sh.kch == 2) launch_grid<2, 2>(P, nb, d_count, d_T, precision, pairs, s);
  else if (sh.kp == 2 && sh.kch == 4) launch_grid<2, 4>(P, nb, d_count, d_T, precision, pairs, s);
  else if (sh.kp == 8 && sh.kch == 1) launch_grid<8, 1>(P, nb, d_count, d_T, precision, pairs, s);
  else if (sh.kp == 8 && sh.kch == 2) launch_grid<8, 2>(P, nb, d_count, d_T, precision, pairs, s);
  else launch_grid<4, 2>(P, nb, d_count, d_T, precision, pairs, s);
}

void th_launch_list_sum(const DevProblem& P, const NodeBufView& nb, const int* d_count, const int64_t* d_pts,
                        int64_t n, double* d_T, int precision, unsigned long long* pairs, cudaStream_t s) {
  if (n <= 0) return;
  const int64_t blocks = (n + kThreads - 1) / kThreads;
  if (precision == 0) k_list_fp64<<<(unsigned)blocks, kThreads, 0, s>>>(P, nb, d_count, d_pts, n, d_T, pairs);
  else k_list_fp32<<<(unsigned)blocks, kThreads, 0, s>>>(P, nb, d_count, d_pts, n, d_T, pairs);
}

void th_launch_nodes_export(const NodeBufView& nb, const int* d_count, double* d_out, int cap, cudaStream_t s) {
  k_nodes_export<<<64, 256, 0, s>>>(nb, d_count, d_out, cap);
}
