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

// Dynamic shared memory of the list-generating kernels: a GenComp for compressing decks.
__global__ void __launch_bounds__(kGenThreads) k_nodes_block(DevProblem P, double t, int is_sol, NodeBufView nb,
                                                             int* count, int* err) {
  __shared__ GenShared sh;
  extern __shared__ __align__(16) unsigned char gen_dyn[];
  gen_list_block(P, t, is_sol != 0, nb, count, err, sh, P.compress ? (GenComp*)gen_dyn : nullptr);
}

// ---------------------------------------------------------------- whole-grid sums
constexpr int kThreads = 256;
constexpr int kChunk = 256;   // nodes staged in shared memory per pass
constexpr int kCJ = 8;        // tile width along j


// Shared memory of one FP32 grid tile.
struct TileShared {
  float4 A[kChunk], B[kChunk];   // node offsets (x, y, z) and coefficients (kx | ky, kz, w)
  float off[64 + 8 + 64];        // point offsets along i, j, k from the tile centre
};

// One tile of the whole-grid FP32 + Kahan sum.  Tile: CI x 8 columns, TK = KP * KCH layers;
// thread (column, k-chunk) owns KP consecutive k-points, processed two at a time with
// packed FP32x2 arithmetic (the per-pair work is four packed issue slots and one MUFU.EX2).
// Offsets from the tile centre are formed once per tile in FP64 and rounded once, so the
// FP32 differences keep ~1e-7 relative accuracy on the tile's scale; the exponent is exp2
// with -3 log2(e) folded into the node coefficients.
template <int KP, int KCH>
__device__ __forceinline__ void tile_fp32(const DevProblem& P, const NodeBufView& nb, int nn, double* __restrict__ T,
                                          int ti, int tj, int tk, TileShared& sh) {
  static_assert(KP % 2 == 0, "KP must be even");
  constexpr int CI = kThreads / KCH / kCJ, TK = KP * KCH;
  const int tid = threadIdx.x;
  const int kc = tid % KCH, col = tid / KCH, ci = col / kCJ, cj = col % kCJ;
  const int i0 = ti * CI, j0 = tj * kCJ, k0t = tk * TK;
  __syncthreads();
  if (tid < CI + kCJ + TK) {
    double v;
    if (tid < CI) v = coord(P.gx, P.xmin, P.xmax, P.hx, i0 + tid) - coord(P.gx, P.xmin, P.xmax, P.hx, i0 + CI / 2);
    else if (tid < CI + kCJ) v = coord(P.gy, P.ymin, P.ymax, P.hy, j0 + tid - CI) - coord(P.gy, P.ymin, P.ymax, P.hy, j0 + kCJ / 2);
    else v = coord(P.gz, P.zmin, P.zmax, P.hz, k0t + tid - CI - kCJ) - coord(P.gz, P.zmin, P.zmax, P.hz, k0t + TK / 2);
    sh.off[tid] = __double2float_rn(v);
  }
  const double Xo = coord(P.gx, P.xmin, P.xmax, P.hx, i0 + CI / 2);
  const double Yo = coord(P.gy, P.ymin, P.ymax, P.hy, j0 + kCJ / 2);
  const double Zo = coord(P.gz, P.zmin, P.zmax, P.hz, k0t + TK / 2);
  __syncthreads();
  const float px = sh.off[ci], py = sh.off[CI + cj];
  unsigned long long pz2[KP / 2], s2[KP / 2], c2[KP / 2];
#pragma unroll
  for (int h = 0; h < KP / 2; ++h) {
    pz2[h] = pk2(sh.off[CI + kCJ + kc * KP + 2 * h], sh.off[CI + kCJ + kc * KP + 2 * h + 1]);
    s2[h] = 0ull;
    c2[h] = 0ull;
  }
  for (int base = 0; base < nn; base += kChunk) {
    __syncthreads();
    const int idx = base + tid;
    if (idx < nn) {
      sh.A[tid] = make_float4(__double2float_rn(nb.x[idx] - Xo), __double2float_rn(nb.y[idx] - Yo),
                              __double2float_rn(nb.z[idx] - Zo), nb.kx[idx]);
      sh.B[tid] = make_float4(nb.ky[idx], nb.kz[idx], nb.w[idx], 0.f);
    }
    __syncthreads();
    const int m = min(kChunk, nn - base);
#pragma unroll 2
    for (int n = 0; n < m; ++n) {
      const float4 a = sh.A[n], b = sh.B[n];
      const float dx = px - a.x, dy = py - a.y;
      const float exy = fmaf(dy * dy, b.x, dx * dx * a.w);
      const unsigned long long oz = pk2(a.z, a.z), kz = pk2(b.y, b.y), ex = pk2(exy, exy), w = pk2(b.z, b.z);
#pragma unroll
      for (int h = 0; h < KP / 2; ++h) {
        const unsigned long long dz = sub2(pz2[h], oz);
        float e0, e1;
        upk2(fma2(mul2(dz, dz), kz, ex), e0, e1);
        const unsigned long long v = mul2(pk2(ex2_approx(e0), ex2_approx(e1)), w);
        const unsigned long long y = sub2(v, c2[h]);
        const unsigned long long t = add2(s2[h], y);
        c2[h] = sub2(sub2(t, s2[h]), y);
        s2[h] = t;
      }
    }
  }
  const int i = i0 + ci, j = j0 + cj, k0 = k0t + kc * KP;
  if (i < P.nx && j < P.ny) {
    const int64_t row = ((int64_t)i * P.ny + j) * P.nz;
#pragma unroll
    for (int h = 0; h < KP / 2; ++h) {
      float s0, s1, cc0, cc1;
      upk2(s2[h], s0, s1);
      upk2(c2[h], cc0, cc1);
      if (k0 + 2 * h < P.nz) T[row + k0 + 2 * h] = P.T0 + ((double)s0 - (double)cc0);
      if (k0 + 2 * h + 1 < P.nz) T[row + k0 + 2 * h + 1] = P.T0 + ((double)s1 - (double)cc1);
    }
  }
}

template <int KP, int KCH>
__global__ void __launch_bounds__(kThreads) k_grid_fp32(DevProblem P, NodeBufView nb, const int* count,
                                                        double* __restrict__ T, int ntj, int ntk,
                                                        unsigned long long* pairs) {
  __shared__ TileShared sh;
  const int nn = min(*count, nb.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(pairs, (unsigned long long)nn * (unsigned long long)P.pnum);
  const int tile = blockIdx.x;
  const int tk = tile % ntk, tij = tile / ntk, tj = tij % ntj, ti = tij / ntj;
  tile_fp32<KP, KCH>(P, nb, nn, T, ti, tj, tk, sh);
}

// Plain FP64 (the reference's arithmetic, one libdevice exp per pair).
template <int KP, int KCH>
__device__ __forceinline__ void tile_fp64(const DevProblem& P, const NodeBufView& nb, int nn, double* __restrict__ T,
                                          int ti, int tj, int tk, double2 (*sN)[4]) {
  constexpr int CI = kThreads / KCH / kCJ, TK = KP * KCH;
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
  __syncthreads();
  if (i < P.nx && j < P.ny) {
    const int64_t row = ((int64_t)i * P.ny + j) * P.nz;
#pragma unroll
    for (int q = 0; q < KP; ++q)
      if (k0 + q < P.nz) T[row + k0 + q] = P.T0 + s[q];
  }
}

template <int KP, int KCH>
__global__ void __launch_bounds__(kThreads) k_grid_fp64(DevProblem P, NodeBufView nb, const int* count,
                                                        double* __restrict__ T, int ntj, int ntk,
                                                        unsigned long long* pairs) {
  __shared__ double2 sN[kChunk][4];
  const int nn = min(*count, nb.cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(pairs, (unsigned long long)nn * (unsigned long long)P.pnum);
  const int tile = blockIdx.x;
  const int tk = tile % ntk, tij = tile / ntk, tj = tij % ntj, ti = tij / ntj;
  tile_fp64<KP, KCH>(P, nb, nn, T, ti, tj, tk, sN);
}

// ---------------------------------------------------------------- batched decks
// Many independent decks in one launch: one block per deck builds its node list...
__global__ void __launch_bounds__(kGenThreads) k_batch_nodes(const DevProblem* probs, const NodeBufView* views,
                                                             const double* times, int* counts, int* err) {
  __shared__ GenShared sh;
  extern __shared__ __align__(16) unsigned char gen_dyn[];
  const int d = blockIdx.x;
  gen_list_block(probs[d], times[d], false, views[d], counts + d, err, sh, (GenComp*)gen_dyn);
}

// ...then a persistent grid drains one work list of (deck, tile) items, taken in order with
// an atomic ticket, so decks of very different sizes and node counts share the SMs.
template <int KP, int KCH, int PREC>
__global__ void __launch_bounds__(kThreads) k_batch_grid(const DevProblem* probs, const NodeBufView* views,
                                                         const int* counts, double* __restrict__ T,
                                                         const long long* pnum_off, const int* tile_off, int ndeck,
                                                         int* ticket, unsigned long long* pairs) {
  constexpr int CI = kThreads / KCH / kCJ, TK = KP * KCH;
  __shared__ TileShared sh;
  __shared__ double2 sN[PREC == 0 ? kChunk : 1][4];
  __shared__ int s_item;
  const int total = tile_off[ndeck];
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(ticket, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    int lo = 0, hi = ndeck - 1;                            // deck of this item
    while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (tile_off[mid] <= item) lo = mid; else hi = mid - 1; }
    const DevProblem& P = probs[lo];
    const NodeBufView nb = views[lo];
    const int nn = min(counts[lo], nb.cap);
    const int tile = item - tile_off[lo];
    const int ntj = (P.ny + kCJ - 1) / kCJ, ntk = (P.nz + TK - 1) / TK;
    const int tk = tile % ntk, tij = tile / ntk, tj = tij % ntj, ti = tij / ntj;
    if (tile == 0 && threadIdx.x == 0) atomicAdd(pairs, (unsigned long long)nn * (unsigned long long)P.pnum);
    if (PREC == 0) tile_fp64<KP, KCH>(P, nb, nn, T + pnum_off[lo], ti, tj, tk, sN);
    else tile_fp32<KP, KCH>(P, nb, nn, T + pnum_off[lo], ti, tj, tk, sh);
    (void)CI;
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
  if (live) point_xyz(P, pts ? pts[gi] : gi, x, y, z);   // pts null: points 0 .. n - 1
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
  if (live) point_xyz(P, pts ? pts[gi] : gi, x, y, z);   // pts null: points 0 .. n - 1
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
  k_nodes_block<<<1, kGenThreads, P.compress ? sizeof(GenComp) : 0, s>>>(P, t, is_sol ? 1 : 0, nb, d_count, d_err);
}

bool th_tile_shape_supported(TileShape sh) {
  return (sh.kp == 4 && (sh.kch == 1 || sh.kch == 2 || sh.kch == 4)) || (sh.kp == 2 && (sh.kch == 2 || sh.kch == 4)) ||
         (sh.kp == 8 && (sh.kch == 1 || sh.kch == 2));
}

void th_launch_grid_sum(const DevProblem& P, const NodeBufView& nb, const int* d_count, double* d_T, int precision,
                        TileShape sh, unsigned long long* pairs, cudaStream_t s) {
  // custom points have no grid to tile: every point as a list
  if (P.cx) { th_launch_list_sum(P, nb, d_count, nullptr, P.pnum, d_T, precision, pairs, s); return; }
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

int th_tile_count(const DevProblem& P, TileShape sh) {
  const int CI = kThreads / sh.kch / kCJ, TK = sh.kp * sh.kch;
  return ((P.nx + CI - 1) / CI) * ((P.ny + kCJ - 1) / kCJ) * ((P.nz + TK - 1) / TK);
}

void th_launch_batch_nodes(int ndeck, const DevProblem* probs, const NodeBufView* views, const double* times,
                           int* counts, int* err, cudaStream_t s) {
  k_batch_nodes<<<ndeck, kGenThreads, sizeof(GenComp), s>>>(probs, views, times, counts, err);
}

template <int KP, int KCH>
static void launch_batch_t(int precision, int blocks, const DevProblem* probs, const NodeBufView* views,
                           const int* counts, double* T, const long long* pnum_off, const int* tile_off, int ndeck,
                           int* ticket, unsigned long long* pairs, cudaStream_t s) {
  if (precision == 0)
    k_batch_grid<KP, KCH, 0><<<blocks, kThreads, 0, s>>>(probs, views, counts, T, pnum_off, tile_off, ndeck, ticket, pairs);
  else
    k_batch_grid<KP, KCH, 1><<<blocks, kThreads, 0, s>>>(probs, views, counts, T, pnum_off, tile_off, ndeck, ticket, pairs);
}

void th_launch_batch_grid(TileShape sh, int precision, const DevProblem* probs, const NodeBufView* views,
                          const int* counts, double* T, const long long* pnum_off, const int* tile_off, int ndeck,
                          int* ticket, unsigned long long* pairs, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 6;
#define TH_BATCH(KP, KCH) launch_batch_t<KP, KCH>(precision, blocks, probs, views, counts, T, pnum_off, tile_off, ndeck, ticket, pairs, s)
  if (sh.kp == 4 && sh.kch == 1) TH_BATCH(4, 1);
  else if (sh.kp == 4 && sh.kch == 4) TH_BATCH(4, 4);
  else if (sh.kp == 2 && sh.kch == 2) TH_BATCH(2, 2);
  else if (sh.kp == 2 && sh.kch == 4) TH_BATCH(2, 4);
  else if (sh.kp == 8 && sh.kch == 1) TH_BATCH(8, 1);
  else if (sh.kp == 8 && sh.kch == 2) TH_BATCH(8, 2);
  else TH_BATCH(4, 2);
#undef TH_BATCH
}

void th_launch_nodes_export(const NodeBufView& nb, const int* d_count, double* d_out, int cap, cudaStream_t s) {
  k_nodes_export<<<64, 256, 0, s>>>(nb, d_count, d_out, cap);
}
