// Solidification mode on the device: windows of per-step node lists, the persistent
// Volume / Surface tracking loop, the NoTracking step, and bulk solidification.
//
// Reference behaviour restated here (3DThesis tree):
//   Run::Solidify_NoTracking / _Volume / _Surface   src/Run.cpp:409-709
//   Melt::beam_trace (+ perimeter)                  src/Melt.cpp:20-183
//   Melt::neighbor_check                            src/Melt.cpp:185-269
//   Melt::calc_depth / calc_depth_max               src/Melt.cpp:271-357
//   Grid::Solidify and the primary solidification   src/Grid.cpp:316-453, 522-548
//
// The reference grows its melt pool with per-point OpenMP locks; here every point owns a
// claim flag taken with atomicCAS, so the sets of evaluated, liquid and solidified points
// are the same whatever order the claims happen in.  Liquid -> solid transitions are
// queued as (point, step, T, T_last) records and their solidification time and gradients
// are computed afterwards, in bulk, one thread per record.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cstdint>
#include <cstdlib>
#include <cuda_runtime.h>

#include "th_device.cuh"
#include "th_track.h"

using namespace thdev;

namespace {

// One slot's node arrays as two base pointers: a window keeps each of its eight double
// fields (x, y, z, ipx, ipy, ipz, dtau, amp) and ten float fields (kx, ky, kz, w, xh, xl, yh,
// yl, zh, zl) in one array of `stride` entries, those arrays `stride` apart, slots one after
// another (window_layout_ok checks this before a launch).  The tracking loop carries two of
// these instead of two full views.
struct SlotRef {
  const double* d;
  const float* f;
  int stride;
  __device__ __forceinline__ double dv(int field, int n) const { return __ldg(d + (size_t)field * stride + n); }
  __device__ __forceinline__ float fv(int field, int n) const { return __ldg(f + (size_t)field * stride + n); }
};
enum { ND_X, ND_Y, ND_Z, ND_IPX, ND_IPY, ND_IPZ, ND_DTAU, ND_AMP };
enum { NF_KX, NF_KY, NF_KZ, NF_W, NF_XH, NF_XL, NF_YH, NF_YL, NF_ZH, NF_ZL };

__device__ __forceinline__ SlotRef slot_ref(const NodeWindow& w, int slot) {
  const size_t off = (size_t)slot * w.slot_cap;
  return SlotRef{w.nb.x + off, w.nb.kx + off, w.nb.cap};
}

// ------------------------------------------------------------------ warp evaluation
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// A step's node list staged in shared memory, one copy per block.  FP32: ten float arrays
// of cap entries (xh, yh, zh, xl, yl, zl, kx, ky, kz, w), read as 16-byte groups of four
// consecutive nodes, the list's zero-weight padding included; FP64: four double2 arrays
// (x, y), (z, 1/phix), (1/phiy, 1/phiz), (dtau, amp).  Nodes at and beyond n_sm are read
// from the window in global memory.
struct Staged {
  const unsigned char* base;
  int n_sm;                // staged nodes
  int cap;                 // nodes per staged array (a multiple of kListPad)
};

template <int PREC>
__host__ __device__ constexpr int staged_bytes_per_node() { return PREC == 0 ? 64 : 40; }

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Issues the block's asynchronous copies of the first m nodes of nb into buf.  FP32 copies
// the list with its zero-weight padding to a multiple of kListPad nodes, in 16-byte groups
// of four (a slot's arrays start 128-byte aligned and hold a multiple of kListPad nodes, and
// cap is a multiple of kListPad, so the padding stays inside both).
template <int PREC>
__device__ __forceinline__ void stage_issue(const NodeBufView& nb, int m, unsigned char* buf, int cap) {
  if (PREC == 0) {
    const double* src[8] = {nb.x, nb.y, nb.z, nb.ipx, nb.ipy, nb.ipz, nb.dtau, nb.amp};
#pragma unroll
    for (int f = 0; f < 8; ++f) {
      double* dst = (double*)(buf + (size_t)(f >> 1) * cap * 16) + (f & 1);
      for (int n = threadIdx.x; n < m; n += blockDim.x) cp_async8(dst + 2 * n, src[f] + n);
    }
  } else {
    const float* src[10] = {nb.xh, nb.yh, nb.zh, nb.xl, nb.yl, nb.zl, nb.kx, nb.ky, nb.kz, nb.w};
    const int groups = min((m + kListPad - 1) & ~(kListPad - 1), cap) >> 2;   // with the list's padding
#pragma unroll
    for (int f = 0; f < 10; ++f) {
      float* dst = (float*)(buf + (size_t)f * cap * 4);
      for (int g = threadIdx.x; g < groups; g += blockDim.x) cp_async16(dst + 4 * g, src[f] + 4 * g);
    }
  }
  cp_async_commit();
}


// One evaluation's result: T as stored (a double in FP64 runs; in FP32 runs the sum T - T0
// as a double-float pair (hi, lo) in the double's bits, decoded by t_decode), and T >= T_L.
struct EvalT { double T; bool liquid; };

// (hi, lo) packed for storage; a zero sum is stored with lo = -0 so that all-zero bits keep
// meaning "never evaluated".
__device__ __forceinline__ double pack_df(float hi, float lo) {
  const unsigned l = (hi == 0.f && lo == 0.f) ? 0x80000000u : __float_as_uint(lo);
  return __longlong_as_double((long long)(((unsigned long long)__float_as_uint(hi) << 32) | l));
}

__device__ __forceinline__ unsigned udiv(unsigned x, unsigned m, int sh) {
  return (unsigned)(((unsigned long long)x * m) >> sh);
}

// (hi, lo) += (bh, bl) in double-float without renormalising: TwoSum of the heads (Knuth),
// the error and both tails summed into lo.  Chained in the lane butterfly, with one
// Fast2Sum (Dekker) at the end.  The result depends only on the two operands as a set
// (TwoSum's error term is exact either way), so both lanes of a butterfly get the same bits.
__device__ __forceinline__ void df_add_lazy(float& hi, float& lo, float bh, float bl) {
  const float s = hi + bh;
  const float v = s - hi;
  lo = ((hi - (s - v)) + (bh - v)) + (lo + bl);
  hi = s;
}

// The FP32 form takes the liquid decision (T >= T_L) on its own sum except within
// kGuardRel (T_L - T_0) of T_L (2 mK on the benchmark decks).  There the point's sum is taken
// again in FP64 from the node window's FP64 fields and decides, exactly as the FP64 form
// decides.  The FP32 sums' error stays below 2.2e-7 of T - T_0 (the largest over every
// evaluated point of the benchmark decks; 1.9e-4 K at their liquidus), seven times inside
// the band, so the molten-point set, and with it every later claim and evaluation, is the
// FP64 form's.  The check sits where a decision is used (guard_T), not in the evaluation
// pass: inside the pass it cost a fifth of the pass's time.  An FP64 pass costs about 20 us
// on this GPU, so the band is kept narrow: about one decision in 70 timesteps takes it.
constexpr float kGuardRel = 1.5e-6f;

// FP64 sum of grid point p over a list's first nn nodes in global memory (the fields of a
// SlotRef: x y z 1/phix 1/phiy 1/phiz dtau amp, `stride` apart), the lanes splitting the
// nodes as the FP64 tracking pass does; every lane returns the sum.  Warp-collective.  The
// point's FP64 coordinates are formed in here from its index: FP64 instructions are slow on
// this GPU, and arguments formed at the call site would be computed on every pass.
__device__ __noinline__ double warp_sum_fp64_point(const double* d, int stride, int nn, unsigned p, unsigned ny,
                                                   unsigned nz, int gx, int gy, int gz, double xmin, double xmax,
                                                   double hx, double ymin, double ymax, double hy, double zmin,
                                                   double zmax, double hz) {
  const int lane = threadIdx.x & 31;
  const unsigned c = p / nz, pk = p - c * nz, pi = c / ny, pj = c - pi * ny;
  const double x = coord(gx, xmin, xmax, hx, (int)pi), y = coord(gy, ymin, ymax, hy, (int)pj),
               z = coord(gz, zmin, zmax, hz, (int)pk);
  double s = 0.0;
  for (int n = lane; n < nn; n += 32) {
    const double dx = x - __ldg(d + n), dy = y - __ldg(d + stride + n), dz = z - __ldg(d + 2 * (size_t)stride + n);
    const double wa = __ldg(d + 6 * (size_t)stride + n) * __ldg(d + 7 * (size_t)stride + n);
    s += wa * exp(-3.0 * (dx * dx * __ldg(d + 3 * (size_t)stride + n) + dy * dy * __ldg(d + 4 * (size_t)stride + n) +
                          dz * dz * __ldg(d + 5 * (size_t)stride + n)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// T at NP points of one grid column (the same i, j; the callers' passes - a point and the
// layers under it, or a run of layers of a depth walk - always are) from one node list,
// the 32 lanes of a warp splitting the nodes; every lane returns the same values.  Each node
// is read once for all NP points, so a pass over four points costs little more than a pass
// over one.
//
// FP32 form: the points' coordinates come as (hi, lo) float pairs from per-axis tables
// (`ax`, in shared memory when it fits); each lane takes groups of four staged nodes (the
// lists are padded with zero-weight nodes to a multiple of 128) as two packed pairs, forms
// the x, y part of the exponent once per node and the z part per point, adds the two
// pairs' terms and folds them into a packed Kahan sum.  The lanes' results are reduced as
// double-float pairs, and the liquid test compares that pair with T_L - T_0 split into
// three floats.  No FP64 arithmetic or conversion sits on the evaluation's path: T is
// stored as the pair and turned into a double only where fields and solidification times
// are computed.
template <int PREC, int NP>
__device__ __forceinline__ void warp_T_n(const DevProblem& P, const TrackState& S, const float2* ax,
                                         const SlotRef& nb, int nn, const int (&pts)[NP], const Staged& st,
                                         EvalT (&out)[NP]) {
  const int lane = threadIdx.x & 31;
  const int n_sm = min(st.n_sm, nn);
  if constexpr (PREC == 0) {
    double x[NP], y[NP], z[NP], s[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const unsigned pu = (unsigned)pts[q], col = pu / (unsigned)P.nz;
      const unsigned pk = pu - col * (unsigned)P.nz, pi = col / (unsigned)P.ny, pj = col - pi * (unsigned)P.ny;
      x[q] = coord(P.gx, P.xmin, P.xmax, P.hx, (int)pi);
      y[q] = coord(P.gy, P.ymin, P.ymax, P.hy, (int)pj);
      z[q] = coord(P.gz, P.zmin, P.zmax, P.hz, (int)pk);
      s[q] = 0.0;
    }
    const double2* D = (const double2*)st.base;
    auto acc = [&](double2 a, double2 b, double2 c, double2 d) {
      const double wa = d.x * d.y;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const double dx = x[q] - a.x, dy = y[q] - a.y, dz = z[q] - b.x;
        s[q] += wa * exp(-3.0 * (dx * dx * b.y + dy * dy * c.x + dz * dz * c.y));
      }
    };
    int n = lane;
    for (; n < n_sm; n += 32) acc(D[n], D[st.cap + n], D[2 * st.cap + n], D[3 * st.cap + n]);
    for (; n < nn; n += 32)
      acc(make_double2(nb.dv(ND_X, n), nb.dv(ND_Y, n)), make_double2(nb.dv(ND_Z, n), nb.dv(ND_IPX, n)),
          make_double2(nb.dv(ND_IPY, n), nb.dv(ND_IPZ, n)), make_double2(nb.dv(ND_DTAU, n), nb.dv(ND_AMP, n)));
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      out[q].T = P.T0 + warp_sum_d(s[q]);
      out[q].liquid = out[q].T >= P.TL;
    }
  } else {
    const unsigned col = udiv((unsigned)pts[0], P.div_nz_m, P.div_nz_s);
    const unsigned pi = udiv(col, P.div_ny_m, P.div_ny_s), pj = col - pi * (unsigned)P.ny;
    const float2 X = ax[pi], Y = ax[P.nx + pj];
    const unsigned long long Xh = pk2(X.x, X.x), Xl = pk2(X.y, X.y), Yh = pk2(Y.x, Y.x), Yl = pk2(Y.y, Y.y);
    // per point its z as (v, v) pairs and one packed Kahan sum (s2, c2) over node pairs (the
    // pairs' even nodes in the low half, odd in the high)
    unsigned long long Zh[NP], Zl[NP], s2[NP], c2[NP];
    float zh1[NP], zl1[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const unsigned pk = min((unsigned)pts[q] - col * (unsigned)P.nz, (unsigned)P.nz - 1u);
      const float2 Z = ax[P.nx + P.ny + pk];
      zh1[q] = Z.x; zl1[q] = Z.y;
      Zh[q] = pk2(Z.x, Z.x); Zl[q] = pk2(Z.y, Z.y);
      s2[q] = c2[q] = 0ull;
    }
    const int cap4 = st.cap >> 2;
    const ulonglong2* F = (const ulonglong2*)st.base;   // field f, group g of four nodes: F[f * cap4 + g]
    // whole padded list: a multiple of 32 groups, the same number for every lane (a warp
    // whose lanes left the loop at different rounds would run the last round as a separate,
    // serialised path)
    const int ng = ((n_sm + kListPad - 1) & ~(kListPad - 1)) >> 2;
    for (int g = lane; g < ng; g += 32) {
      const ulonglong2 xh = F[g], yh = F[cap4 + g], zh = F[2 * cap4 + g], xl = F[3 * cap4 + g],
                       yl = F[4 * cap4 + g], zl = F[5 * cap4 + g], kx = F[6 * cap4 + g], ky = F[7 * cap4 + g],
                       kz = F[8 * cap4 + g], w = F[9 * cap4 + g];
      const unsigned long long dxa = add2(sub2(Xh, xh.x), sub2(Xl, xl.x)), dxb = add2(sub2(Xh, xh.y), sub2(Xl, xl.y));
      const unsigned long long dya = add2(sub2(Yh, yh.x), sub2(Yl, yl.x)), dyb = add2(sub2(Yh, yh.y), sub2(Yl, yl.y));
      const unsigned long long ea = fma2(mul2(dya, dya), ky.x, mul2(mul2(dxa, dxa), kx.x));
      const unsigned long long eb = fma2(mul2(dyb, dyb), ky.y, mul2(mul2(dxb, dxb), kx.y));
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const unsigned long long dza = add2(sub2(Zh[q], zh.x), sub2(Zl[q], zl.x));
        const unsigned long long dzb = add2(sub2(Zh[q], zh.y), sub2(Zl[q], zl.y));
        const unsigned long long fa = fma2(mul2(dza, dza), kz.x, ea), fb = fma2(mul2(dzb, dzb), kz.y, eb);
        float a0, a1, b0, b1;
        upk2(fa, a0, a1);
        upk2(fb, b0, b1);
        const unsigned long long va = mul2(pk2(ex2_approx(a0), ex2_approx(a1)), w.x);
        const unsigned long long vb = mul2(pk2(ex2_approx(b0), ex2_approx(b1)), w.y);
        const unsigned long long y = sub2(add2(va, vb), c2[q]);
        const unsigned long long t = add2(s2[q], y);
        c2[q] = sub2(sub2(t, s2[q]), y);
        s2[q] = t;
      }
    }
    float hi[NP], lo[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      float sl, sh, cl, ch;
      upk2(s2[q], sl, sh);
      upk2(c2[q], cl, ch);
      hi[q] = sl;
      lo[q] = -cl;
      df_add_lazy(hi[q], lo[q], sh, -ch);
    }
    if (n_sm < nn) {                               // nodes past the staged copy, one per lane
      float s1[NP], c1[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) s1[q] = c1[q] = 0.f;
      for (int n = n_sm + lane; n < nn; n += 32) {
        const float xh = nb.fv(NF_XH, n), yh = nb.fv(NF_YH, n), zh = nb.fv(NF_ZH, n), xl = nb.fv(NF_XL, n),
                    yl = nb.fv(NF_YL, n), zl = nb.fv(NF_ZL, n), kx = nb.fv(NF_KX, n), ky = nb.fv(NF_KY, n),
                    kz = nb.fv(NF_KZ, n), w = nb.fv(NF_W, n);
        const float dx = (X.x - xh) + (X.y - xl), dy = (Y.x - yh) + (Y.y - yl);
        const float exy = fmaf(dy * dy, ky, dx * dx * kx);
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const float dz = (zh1[q] - zh) + (zl1[q] - zl);
          const float v = ex2_approx(fmaf(dz * dz, kz, exy)) * w;
          const float yy = v - c1[q];
          const float tt = s1[q] + yy;
          c1[q] = (tt - s1[q]) - yy;
          s1[q] = tt;
        }
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) df_add_lazy(hi[q], lo[q], s1[q], -c1[q]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float bh = __shfl_xor_sync(0xffffffffu, hi[q], o), bl = __shfl_xor_sync(0xffffffffu, lo[q], o);
        df_add_lazy(hi[q], lo[q], bh, bl);
      }
    }
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const float sh = hi[q];                      // Fast2Sum: |lo| is far below |hi|
      hi[q] = sh + lo[q];
      lo[q] = lo[q] - (hi[q] - sh);
      // sign of (hi + lo) - (T_L - T_0): the head difference is exact near the threshold
      const float d = ((hi[q] - P.tl_df[0]) + (lo[q] - P.tl_df[1])) - P.tl_df[2];
      out[q].liquid = d >= 0.f;
      out[q].T = pack_df(hi[q], lo[q]);
    }
  }
}

// T at NP points anywhere on the grid (Volume tracking's batches: a chunk of re-tests, or the
// neighbours one item claimed) from one node list, every lane returning the same values.
// FP64: warp_T_n, whose FP64 form takes each point's own coordinates.  FP32: warp_T_n's
// arithmetic with the x and y parts formed per point instead of once per column, so each
// point's sum is bit for bit the one a pass over that point alone gives; the NP points'
// independent sums are what keep a lane's pipes busy.
template <int PREC, int NP>
__device__ __forceinline__ void warp_T_gen(const DevProblem& P, const TrackState& S, const float2* ax,
                                           const SlotRef& nb, int nn, const int (&pts)[NP], const Staged& st,
                                           EvalT (&out)[NP]) {
  if constexpr (PREC == 0) {
    warp_T_n<0, NP>(P, S, ax, nb, nn, pts, st, out);
  } else {
    const int lane = threadIdx.x & 31;
    const int n_sm = min(st.n_sm, nn);
    unsigned long long Xh[NP], Xl[NP], Yh[NP], Yl[NP], Zh[NP], Zl[NP], s2[NP], c2[NP];
    // a point's axis-table entries (coordinates as (hi, lo) floats); looked up again for the
    // rare nodes past the staged copy rather than kept live through the pass
    auto axes = [&](int q, float2& X, float2& Y, float2& Z) {
      const unsigned col = udiv((unsigned)pts[q], P.div_nz_m, P.div_nz_s);
      const unsigned pi = udiv(col, P.div_ny_m, P.div_ny_s), pj = col - pi * (unsigned)P.ny;
      const unsigned pk = min((unsigned)pts[q] - col * (unsigned)P.nz, (unsigned)P.nz - 1u);
      X = ax[pi]; Y = ax[P.nx + pj]; Z = ax[P.nx + P.ny + pk];
    };
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      float2 X, Y, Z;
      axes(q, X, Y, Z);
      Xh[q] = pk2(X.x, X.x); Xl[q] = pk2(X.y, X.y);
      Yh[q] = pk2(Y.x, Y.x); Yl[q] = pk2(Y.y, Y.y);
      Zh[q] = pk2(Z.x, Z.x); Zl[q] = pk2(Z.y, Z.y);
      s2[q] = c2[q] = 0ull;
    }
    const int cap4 = st.cap >> 2;
    const ulonglong2* F = (const ulonglong2*)st.base;
    const int ng = ((n_sm + kListPad - 1) & ~(kListPad - 1)) >> 2;
    for (int g = lane; g < ng; g += 32) {
      const ulonglong2 xh = F[g], yh = F[cap4 + g], zh = F[2 * cap4 + g], xl = F[3 * cap4 + g],
                       yl = F[4 * cap4 + g], zl = F[5 * cap4 + g], kx = F[6 * cap4 + g], ky = F[7 * cap4 + g],
                       kz = F[8 * cap4 + g], w = F[9 * cap4 + g];
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const unsigned long long dxa = add2(sub2(Xh[q], xh.x), sub2(Xl[q], xl.x));
        const unsigned long long dxb = add2(sub2(Xh[q], xh.y), sub2(Xl[q], xl.y));
        const unsigned long long dya = add2(sub2(Yh[q], yh.x), sub2(Yl[q], yl.x));
        const unsigned long long dyb = add2(sub2(Yh[q], yh.y), sub2(Yl[q], yl.y));
        const unsigned long long ea = fma2(mul2(dya, dya), ky.x, mul2(mul2(dxa, dxa), kx.x));
        const unsigned long long eb = fma2(mul2(dyb, dyb), ky.y, mul2(mul2(dxb, dxb), kx.y));
        const unsigned long long dza = add2(sub2(Zh[q], zh.x), sub2(Zl[q], zl.x));
        const unsigned long long dzb = add2(sub2(Zh[q], zh.y), sub2(Zl[q], zl.y));
        const unsigned long long fa = fma2(mul2(dza, dza), kz.x, ea), fb = fma2(mul2(dzb, dzb), kz.y, eb);
        float a0, a1, b0, b1;
        upk2(fa, a0, a1);
        upk2(fb, b0, b1);
        const unsigned long long va = mul2(pk2(ex2_approx(a0), ex2_approx(a1)), w.x);
        const unsigned long long vb = mul2(pk2(ex2_approx(b0), ex2_approx(b1)), w.y);
        const unsigned long long y = sub2(add2(va, vb), c2[q]);
        const unsigned long long t = add2(s2[q], y);
        c2[q] = sub2(sub2(t, s2[q]), y);
        s2[q] = t;
      }
    }
    float hi[NP], lo[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      float sl, sh, cl, ch;
      upk2(s2[q], sl, sh);
      upk2(c2[q], cl, ch);
      hi[q] = sl;
      lo[q] = -cl;
      df_add_lazy(hi[q], lo[q], sh, -ch);
    }
    if (n_sm < nn) {                               // nodes past the staged copy, one per lane
      float s1[NP], c1[NP], x1[NP][2], y1[NP][2], z1[NP][2];
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        s1[q] = c1[q] = 0.f;
        float2 X, Y, Z;
        axes(q, X, Y, Z);
        x1[q][0] = X.x; x1[q][1] = X.y; y1[q][0] = Y.x; y1[q][1] = Y.y; z1[q][0] = Z.x; z1[q][1] = Z.y;
      }
      for (int n = n_sm + lane; n < nn; n += 32) {
        const float xh = nb.fv(NF_XH, n), yh = nb.fv(NF_YH, n), zh = nb.fv(NF_ZH, n), xl = nb.fv(NF_XL, n),
                    yl = nb.fv(NF_YL, n), zl = nb.fv(NF_ZL, n), kx = nb.fv(NF_KX, n), ky = nb.fv(NF_KY, n),
                    kz = nb.fv(NF_KZ, n), w = nb.fv(NF_W, n);
#pragma unroll
        for (int q = 0; q < NP; ++q) {
          const float dx = (x1[q][0] - xh) + (x1[q][1] - xl), dy = (y1[q][0] - yh) + (y1[q][1] - yl);
          const float exy = fmaf(dy * dy, ky, dx * dx * kx);
          const float dz = (z1[q][0] - zh) + (z1[q][1] - zl);
          const float v = ex2_approx(fmaf(dz * dz, kz, exy)) * w;
          const float yy = v - c1[q];
          const float tt = s1[q] + yy;
          c1[q] = (tt - s1[q]) - yy;
          s1[q] = tt;
        }
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) df_add_lazy(hi[q], lo[q], s1[q], -c1[q]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const float bh = __shfl_xor_sync(0xffffffffu, hi[q], o), bl = __shfl_xor_sync(0xffffffffu, lo[q], o);
        df_add_lazy(hi[q], lo[q], bh, bl);
      }
    }
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const float sh = hi[q];
      hi[q] = sh + lo[q];
      lo[q] = lo[q] - (hi[q] - sh);
      const float d = ((hi[q] - P.tl_df[0]) + (lo[q] - P.tl_df[1])) - P.tl_df[2];
      out[q].liquid = d >= 0.f;
      out[q].T = pack_df(hi[q], lo[q]);
    }
  }
}

// a[i] of a four-entry register array without local-memory indexing.
__device__ __forceinline__ EvalT pick4(const EvalT (&a)[4], int i) {
  return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

// T from its stored form (see EvalT); 0 is a point never evaluated (the reference's
// zero-initialised grid).
__device__ __forceinline__ double t_decode(const TrackState& S, const DevProblem& P, double raw) {
  if (!S.t_fixed) return raw;
  const unsigned long long b = (unsigned long long)__double_as_longlong(raw);
  if (b == 0ull) return 0.0;
  return P.T0 + ((double)__uint_as_float((unsigned)(b >> 32)) + (double)__uint_as_float((unsigned)b));
}

__device__ __forceinline__ int ldcg_i(const int* p) { return __ldcg(p); }
__device__ __forceinline__ double ldcg_d(const double* p) { return __ldcg(p); }

__device__ __forceinline__ int push_record(const TrackState& S, int p, int step, double t, double T, double Tl) {
  const int i = atomicAdd(S.rec_n, 1);
  if (i < S.rec_cap) { SolRec r; r.p = p; r.step = step; r.t = t; r.T = T; r.Tl = Tl; S.rec[i] = r; }
  else atomicOr(S.err, ERR_RECORDS);
  atomicAdd(&S.num_melt[p], 1);
  return i;
}

// A block's solidification records, gathered in shared memory and appended to the launch's
// record buffer when half full and at the end of the launch (one atomic per flush), so
// items never wait on the global record counter.  A full buffer falls back to the global
// list.
constexpr int kBlkRec = 256;
struct BlockBuf {
  int nrec, base_rec;
  SolRec rec[kBlkRec];
};

// The step word of QueueCounters::state.  Volume: items completed (bits 0-23), items
// published (24-47), blocks that have entered the step (48-63).  Surface forms: completed
// (0-17), published (18-35), the step's liquid points (36-53), blocks entered (54-62) and a
// request to end the launch after the step (63), so that a waiting warp learns from this
// one word that the step is over, how long the next step's list is and the launch's verdict.
constexpr int kSurfLiq = 36;
constexpr unsigned long long kSurfStop = 1ull << 63;
template <bool SURF>
struct StepWord {
  static constexpr int kPub = SURF ? 18 : 24, kArr = SURF ? 54 : 48;
  static constexpr unsigned long long kField = SURF ? 0x3ffffull : 0xffffffull;
  static constexpr unsigned long long kArrMask = SURF ? 0x1ffull : 0xffffull;
  static constexpr unsigned long long kArrive = 1ull << kArr;
  __host__ __device__ static unsigned completed(unsigned long long v) { return (unsigned)(v & kField); }
  __host__ __device__ static unsigned published(unsigned long long v) { return (unsigned)((v >> kPub) & kField); }
  __host__ __device__ static unsigned entered(unsigned long long v) { return (unsigned)((v >> kArr) & kArrMask); }
  __host__ __device__ static unsigned liquid(unsigned long long v) { return (unsigned)((v >> kSurfLiq) & kField); }
  __host__ __device__ static bool over(unsigned long long v, int n_init, unsigned blocks) {
    return entered(v) == blocks && completed(v) == (unsigned long long)n_init + published(v);
  }
};

// Grid::Calc_T with set = true (src/Grid.cpp:300-311): the liquid markers (G = V = DBL_MIN,
// eqFrac = -1) are applied when fields are read, from last_liq.
__device__ __forceinline__ void set_T(const TrackState& S, int p, const EvalT& e, int step) {
  S.T[p] = e.T;
  if (e.liquid) { S.outflag[p] = 1; S.last_liq[p] = step; }
}

// Bound on the polls of one wait for work (seconds: each poll is an L2 round trip after its
// back-off); past it the
// waiter latches ERR_BARRIER and releases every warp of the launch.  The test knob
// THESIS_GB300_SPIN_LIMIT lowers it.
constexpr long long kSpinLimit = 1ll << 25;


__device__ __forceinline__ int64_t pid(const DevProblem& P, int i, int j, int k) {
  return (int64_t)i * ((int64_t)P.ny * P.nz) + (int64_t)j * P.nz + k;
}

// Claim for this step (the reference's T_calc_flag test-and-set, src/Melt.cpp:213-218):
// a point counts as claimed in step k when its stamp is >= k + 1.
__device__ __forceinline__ bool claim(const TrackState& S, int q, unsigned stamp) {
  return atomicMax(S.stamp + q, stamp) < stamp;
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// ------------------------------------------------------------------ step work queue
enum { IT_RETEST = 0, IT_VISIT = 2, IT_COLUMN = 3, IT_EXPAND = 4 };

// Tracking forms of the loop: Volume, Surface, Surface logging RDF melt events, and Stork
// (Surface's search without solidification, which logs the liquid columns for the doubly
// reduced data).  Each is its own instantiation, so a form carries none of the others' work.
enum { TM_VOLUME = 0, TM_SURFACE = 1, TM_STORK = 2, TM_SURFACE_RDF = 3 };

struct StepCtx {
  Staged st, stl;          // this step's and the previous step's node lists in shared memory
  BlockBuf* bb;            // this block's buffered records
  mutable unsigned long long ev_n, ev_c, ev_nodes;  // evaluation passes, their SM clocks and nodes (profile)
  int depth;               // chain depth of the item being run (its children get depth + 1)
  int k;                   // step
  unsigned stamp;          // k + 1
  double t;
  SlotRef nb, nbl;
  int nn, nnl;
  int nL, n_init;
  const int2* L;
  int2* Lo;
  int* lo_n;
  QueueCounters* qc;
  const float2* ax;        // grid axis table (hi, lo) (shared memory when it fits)
  int log_out;             // Stork: where this step's liquid list starts in the launch's log
  int log_j;               // and which of the launch's lists it is
  int hw;                  // the record buffer's high-water mark
  mutable int liq;         // Surface forms: the item joined the next step's list (counted at completion)
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long atom_add_release(unsigned long long* p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.add.release.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_relaxed_v2(ulonglong2* p, unsigned long long a, unsigned long long b) {
  asm volatile("st.relaxed.gpu.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}
__device__ __forceinline__ ulonglong2 ld_relaxed_v2(const ulonglong2* p) {
  ulonglong2 v;
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_or(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.or.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

template <int PREC>
__device__ __forceinline__ EvalT eval_T(const DevProblem& P, const TrackState& S, const StepCtx& X,
                                        const SlotRef& nb, int nn, int64_t p, const Staged& st) {
  const long long c0 = clock64();
  const int pts[1] = {(int)p};
  EvalT T[1];
  warp_T_n<PREC, 1>(P, S, X.ax, nb, nn, pts, st, T);
  X.ev_c += clock64() - c0;
  X.ev_n += 1;
  X.ev_nodes += nn;
  return T[0];
}

// NP points of this step's list in one pass (entries the caller does not need may repeat
// a valid point).
template <int PREC, int NP>
__device__ __forceinline__ void eval_Tn(const DevProblem& P, const TrackState& S, const StepCtx& X,
                                        const int (&pts)[NP], EvalT (&T)[NP]) {
  const long long c0 = clock64();
  warp_T_n<PREC, NP>(P, S, X.ax, X.nb, X.nn, pts, X.st, T);
  X.ev_c += clock64() - c0;
  X.ev_n += 1;
  X.ev_nodes += X.nn;
}

// FP32 runs: an evaluation of point p on this step's list whose sum lies within the guard band of
// T_L takes its liquid decision, and its T, from the FP64 sum instead.  Warp-collective (T
// is the same in every lane); called before the decision is used or stored.
template <int PREC>
__device__ __forceinline__ void guard_T(const DevProblem& P, const TrackState& S, const StepCtx& X, EvalT& T, int p) {
  if (PREC == 0) return;
  const unsigned long long b = (unsigned long long)__double_as_longlong(T.T);
  const float hi = __uint_as_float((unsigned)(b >> 32)), lo = __uint_as_float((unsigned)b);
  const float d = ((hi - P.tl_df[0]) + (lo - P.tl_df[1])) - P.tl_df[2];
  if (fabsf(d) < kGuardRel * P.tl_df[0]) {
    const double s = warp_sum_fp64_point(X.nb.d, X.nb.stride, X.nn, (unsigned)p, (unsigned)P.ny, (unsigned)P.nz,
                                         P.gx, P.gy, P.gz, P.xmin, P.xmax, P.hx, P.ymin, P.ymax, P.hy, P.zmin,
                                         P.zmax, P.hz);
    T.liquid = P.T0 + s >= P.TL;
    const float sh = __double2float_rn(s);
    T.T = pack_df(sh, __double2float_rn(s - (double)sh));
    if ((threadIdx.x & 31) == 0) atomicAdd(&S.C->guard_total, 1ull);
  }
}

// A claimed neighbour the warp keeps instead of publishing it (Volume tracking): it runs in
// the same warp right after the item that claimed it and is part of that item (never
// published, never completed on its own), so it starts without a trip through the queue.
struct Kept { int p, aux; bool valid; };

// Publishes one child item per lane that has one (warp-uniform call); with `keep`, the
// lowest such lane's child is kept instead when the item keeps none yet.  The children are
// counted as published in the same atomic that hands out their slots, before any of them
// can be taken, so "completed == initial + published" can only hold once the step has no
// work left.  Both 64-bit words of a slot carry the step's stamp, so a reader that sees
// the stamp in both has the whole item without any further ordering.
template <bool SURF>
__device__ __forceinline__ void emit(const TrackState& S, const StepCtx& X, bool has, int type, int p, int aux,
                                     int& nchild, Kept* keep = nullptr) {
  using W = StepWord<SURF>;
  const int lane = threadIdx.x & 31;
  unsigned m = __ballot_sync(0xffffffffu, has);
  if (!m) return;
  if (keep != nullptr && !keep->valid) {
    const int kl = __ffs(m) - 1;
    keep->p = __shfl_sync(0xffffffffu, p, kl);
    keep->aux = __shfl_sync(0xffffffffu, aux, kl);
    keep->valid = true;
    m &= m - 1u;
    if (lane == kl) has = false;
    if (!m) return;
  }
  unsigned base = 0;
  if (lane == 0) base = W::published(atomicAdd(&X.qc->state, (unsigned long long)__popc(m) << W::kPub));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (has) {
    const unsigned j = base + __popc(m & ((1u << lane) - 1u));
    if (j < (unsigned)S.queue_cap) {
      const unsigned long long hi = (unsigned long long)X.stamp << 32;
      st_relaxed_v2(S.queue + j, hi | (unsigned)p,
                    hi | (unsigned)(type | (min(X.depth + 1, 255) << 8) | (aux << 16)));
    } else {
      atomicOr(S.err, ERR_QUEUE);
    }
  }
  nchild += __popc(m);
}

// Claims the unvisited neighbours of p (3x3 in the same layer for Surface, 3x3x{k-1, k}
// for Volume; src/Melt.cpp:202-257) and queues them for evaluation.  A Surface neighbour's
// item carries its column's depth, read beside the claim: only that item writes the
// column's depth this step, so the child starts its pass without a load of its own.
// The claims in flight: per lane the neighbour, its column's depth and the stamp the claim
// replaced (the claim took the point if that is below this step's stamp).
struct Claims { int q, dq; unsigned old; };

template <bool SURF>
__device__ __forceinline__ Claims claim_neighbours(const DevProblem& P, const TrackState& S, const StepCtx& X, int p) {
  const int lane = threadIdx.x & 31;
  const int nyz = P.ny * P.nz;
  const int pi = p / nyz, pj = (p / P.nz) % P.ny, pk = p % P.nz;
  Claims c{0, 0, 0xffffffffu};
  if (lane < (SURF ? 9 : 18)) {
    const int di = (lane % 9) / 3 - 1, dj = lane % 3 - 1, dk = SURF ? 0 : (lane / 9) - 1;
    const int ni = pi + di, nj = pj + dj, nk = pk + dk;
    if (!(ni < 0 || ni > P.nx - 1 || nj < 0 || nj > P.ny - 1 || nk < 0)) {
      c.q = (int)pid(P, ni, nj, nk);
      if (SURF) c.dq = ldcg_i(S.depths + (ni * P.ny + nj));
      c.old = atomicMax(S.stamp + c.q, X.stamp);
    }
  }
  return c;
}

template <bool SURF>
__device__ __forceinline__ void emit_claimed(const TrackState& S, const StepCtx& X, const Claims& c, int& nchild,
                                             Kept* keep) {
  emit<SURF>(S, X, c.old < X.stamp, IT_VISIT, c.q, c.dq, nchild, keep);
}

template <bool SURF>
__device__ __forceinline__ void expand(const DevProblem& P, const TrackState& S, const StepCtx& X, int p, int& nchild,
                                       Kept* keep) {
  emit_claimed<SURF>(S, X, claim_neighbours<SURF>(P, S, X, p), nchild, keep);
}

// A liquid point joins the next step's list with its column's depth (the next re-test
// needs both).  The slot is reserved as soon as the point is known to be liquid and filled
// when the item ends, so the reservation's round trip overlaps the item's other work.
__device__ __forceinline__ void push_liquid(const TrackState& S, const StepCtx& X, int i, int p, int depth) {
  atomicMax(S.stamp + p, X.stamp + 1u);   // already claimed for the next step's re-test
  if (i < S.list_cap) X.Lo[i] = make_int2(p, depth); else atomicOr(S.err, ERR_LISTS);
  X.liq = 1;
}

// Stork: the liquid point also joins the launch's log of liquid lists (the doubly reduced
// data is built from it after the launch), at the same index as in the next step's list.
__device__ __forceinline__ void log_liquid(const TrackState& S, const StepCtx& X, int i, int p, int depth) {
  const int j = X.log_out + i;
  if (j < S.rlog_cap) S.rlog[j] = make_int2(p, depth); else atomicOr(S.err, ERR_LISTS);
}

// The counters of a step are cleared while no warp can touch them: those of step k + 1
// (queue and step word, in the third of the rotating sets: last used by step k - 2) and the
// slot counter of the list step k + 1 fills (last used by step k - 2).  Volume: by the lane
// whose update ended step k (every block has entered step k, so none still reads step
// k - 2's counters).  Surface forms: by every block as it enters step k, before its entry
// is counted (all blocks have left step k - 2, and step k + 1 starts only once every block
// has entered step k); the entry is made when the block's first warp has run out of the
// step's initial items.
__device__ __forceinline__ void clear_counters(TrackCounters* C, int k) {
  QueueCounters& q = C->q[(k + 1) % 3];
  q.head = 0; q.depth = 0; q.state = 0ull; q.init_head = 0;
  for (int l = 0; l < 4; ++l) { q.lvl_start[l] = 0; q.lvl_end[l] = 0; }
  C->liq_n[(k + 2) % 3] = 0;
}

// Volume: run by the one lane whose update ended step k: clears the counters, records the
// step, then publishes the step's end.  It also takes the step's verdict for every warp -
// the finish test (src/Util.cpp:239-243) and the record queue's high-water mark, from the
// step's final counts - and publishes it with the next step's liquid-list length and the
// step's stamp in one word, so a waiting warp learns all three from the load that ends its
// wait.
__device__ void finish_step(const DevProblem& P, const TrackState& S, const StepCtx& X, int k, unsigned long long v,
                            int high_water) {
  TrackCounters* C = S.C;
  clear_counters(C, k);
  C->step = k + 1;
  const int items = X.n_init + (int)StepWord<false>::published(v);
  if (items > C->max_items) C->max_items = items;
  const int n_next = __ldcg(X.lo_n), n_rec = __ldcg(S.rec_n);
  unsigned long long flags = 0;
  if (X.t > P.end_time && n_next == 0) { flags |= 1u; C->done = 1; }
  else if (n_rec > high_water) { flags |= 2u; C->stop = 1; }
  // the release store orders this lane's counter resets before the step-end word
  st_release_u64(&C->fin, ((unsigned long long)n_next << 34) | (flags << 32) | X.stamp);
}

// Surface forms: run by the one lane whose update ended the step, v the step word after it.
// The word holds everything the step-end word needs - the next step's list length and a
// stop requested during the step (record buffer or melt-event log past its high-water
// mark) - so the lane publishes the end at once, with the verdict: the finish test
// (src/Util.cpp:239-243), else the stop request or, for Stork, a launch log that could not
// take another whole list.  The counters were cleared as the blocks entered the step, and
// the host's record of the step follows the publication.
template <int TM>
__device__ void surface_finish(const DevProblem& P, const TrackState& S, const StepCtx& X, unsigned long long v) {
  using W = StepWord<true>;
  TrackCounters* C = S.C;
  const unsigned n_next = min(W::liquid(v), (unsigned)S.list_cap);   // more latched ERR_LISTS
  const bool log_full = TM == TM_STORK && (long long)X.log_out + n_next > (long long)S.rlog_cap - S.rlog_step_max;
  unsigned long long flags = 0;
  if (X.t > P.end_time && n_next == 0) flags = 1;
  else if ((v & kSurfStop) || log_full) flags = 2;
  st_release_u64(&C->fin, ((unsigned long long)n_next << 34) | (flags << 32) | X.stamp);
  C->step = X.k + 1;
  atomicMax(&C->max_items, X.n_init + (int)W::published(v));
  if (flags == 1) C->done = 1;
  else if (flags == 2) C->stop = 1;
  if (TM == TM_STORK) S.rlog_off[X.log_j + 1] = X.log_out + n_next;   // the list's end in the launch's log
}

// A record past the buffer's high-water mark asks the Surface forms' step to end the launch.
template <int TM>
__device__ __forceinline__ void push_rec(const TrackState& S, const StepCtx& X, int p, double T, double Tl) {
  if (TM == TM_SURFACE_RDF) S.rdf_open[p] -= 1;       // RDF: a solidification time follows
  const int b = atomicAdd(&X.bb->nrec, 1);
  if (b < kBlkRec) {
    SolRec& r = X.bb->rec[b];
    r.p = p; r.step = X.k; r.t = X.t; r.T = T; r.Tl = Tl;
    atomicAdd(&S.num_melt[p], 1);
  } else {
    const int i = push_record(S, p, X.k, X.t, T, Tl);
    if (TM != TM_VOLUME && i >= X.hw) red_or(&X.qc->state, kSurfStop);
  }
}

// RDF of Surface runs: point q, evaluated liquid in this step, opens a melt event unless
// one is open - the next step's reset sweep pushes t - dt while the point has as many
// melting as solidification times (src/Run.cpp:604-609, src/Grid.h:400-404).  Called by the
// lane that stores q's T, after any solidification of q in the same item (an item is the
// only one to touch its point in a step, so the step's order is kept).
__device__ __forceinline__ void rdf_melt(const TrackState& S, const StepCtx& X, int q) {
  if (S.rdf_open[q] != 0) return;
  S.rdf_open[q] = 1;
  const int j = atomicAdd(S.tm_n, 1);
  if (j < S.tm_cap) S.tm_log[j] = make_int2(q, X.k); else atomicOr(S.err, ERR_RDF);
  if (j >= S.tm_cap / 2) red_or(&X.qc->state, kSurfStop);   // the log's high-water mark
}

// Appends the block's buffered records to the launch's record buffer (all threads of the
// block; ends with the buffer empty).  Returns the launch buffer's length after the append
// as this block's atomic saw it (0 if the block had none; the same in every thread).
__device__ int flush_block(const TrackState& S, BlockBuf* bbp, int* rec_n) {
  BlockBuf& bb = *bbp;
  __syncthreads();
  const int nr = min(bb.nrec, kBlkRec);
  if (threadIdx.x == 0) bb.base_rec = nr ? atomicAdd(rec_n, nr) : 0;
  __syncthreads();
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    const int j = bb.base_rec + i;
    if (j < S.rec_cap) S.rec[j] = bb.rec[i]; else atomicOr(S.err, ERR_RECORDS);
  }
  __syncthreads();
  const int total = nr ? bb.base_rec + nr : 0;
  if (threadIdx.x == 0) bb.nrec = 0;
  __syncthreads();
  return total;
}

// First segment whose end time is >= t, clamped to the last (src/Melt.cpp:58-60), found by
// the whole warp: each round probes 32 evenly spaced segments, so a path of up to 1024
// segments takes two dependent loads instead of ten.  Every lane returns the same index.
__device__ __forceinline__ int warp_first_ge(const DevSeg* path, int ns, double t) {
  const int lane = threadIdx.x & 31;
  int lo = 0, hi = ns - 1;                 // the answer lies in [lo, hi]
  while (lo < hi) {
    const int step = (hi - lo + 32) / 32;  // probes lo, lo + step, ... cover [lo, hi]
    const int idx = min(lo + lane * step, hi);
    const unsigned m = __ballot_sync(0xffffffffu, __ldg(&path[idx].tend) >= t);
    if (m == 0u) { lo = min(lo + 31 * step, hi) + 1; if (lo > hi) lo = hi; continue; }
    const int f = __ffs(m) - 1;
    const int top = min(lo + f * step, hi);
    lo = f == 0 ? lo : min(lo + (f - 1) * step, hi) + 1;
    hi = top;
    if (step == 1) lo = hi;
  }
  return lo;
}

// Surface points of one grid edge within the trace radius of an anchor outside the grid
// (the perimeter lambda of src/Melt.cpp:36-55).  Only points whose distance along the edge
// can be below the radius are tested - a window of +-(r / res + 2) points around the
// anchor's projection - with the reference's exact FP64 test.
template <class Sink>
__device__ void perimeter_edge(const DevProblem& P, bool xfixed, int fixed, double x, double y, double r2,
                               Sink& sink) {
  const int lane = threadIdx.x & 31;
  const int hi = xfixed ? P.ny : P.nx;
  const double c = xfixed ? (y - P.ymin) / P.yres : (x - P.xmin) / P.xres;
  const double w = sqrt(r2) / (xfixed ? P.yres : P.xres) + 2.0;
  const int v_lo = (int)fmin(fmax(0.0, floor(c - w)), (double)hi);
  const int v_hi = (int)fmax(fmin((double)hi, ceil(c + w) + 1.0), 0.0);
  for (int v0 = v_lo; v0 < v_hi; v0 += 32) {
    const int v = v0 + lane;
    bool has = false;
    int q = 0;
    if (v < v_hi) {
      const int i = xfixed ? fixed : v, j = xfixed ? v : fixed;
      const double dx = rn_sub(rn_add(P.xmin, rn_mul((double)i, P.xres)), x);
      const double dy = rn_sub(rn_add(P.ymin, rn_mul((double)j, P.yres)), y);
      if (rn_add(rn_mul(dx, dx), rn_mul(dy, dy)) < r2) { q = (int)pid(P, i, j, P.nz - 1); has = true; }
    }
    sink(has, q);
  }
}

// Melt::beam_trace for (t - dt, t] (src/Melt.cpp:20-183): every surface point the trace
// tests, handed to the sink (warp-collective; claims are taken by the consumer).  The
// anchors of a beam (segment end points in the window, then the beam's position) are
// handled one per lane; perimeter scans (anchors outside the grid, src/Melt.cpp:62-77) and
// the 2 x 2 surface cells at and after anchors inside it (src/Melt.cpp:122-146) follow.
template <class Sink>
__device__ void beam_trace(const DevProblem& P, double t_end, Sink& sink) {
  const int lane = threadIdx.x & 31;
  const double t_start = rn_sub(t_end, P.dt);
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam& B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    const double ts = (rn_sub(t_end, B.tsub) < 0.0) ? 0.0 : rn_sub(t_end, B.tsub);
    const int s1 = warp_first_ge(path, B.nseg, t_end);
    const int s0 = warp_first_ge(path, B.nseg, ts);
    const int c0 = warp_first_ge(path, B.nseg, t_start);
    const bool moving = path[s1].mode == 0 && t_end < B.tlast;
    for (int pass = 0; pass < 2; ++pass) {    // 0: perimeter anchors from ts, 1: cell anchors from t_start
      const int first = max((pass == 0 ? s0 : c0) - 1, 0);
      const int na = s1 - first + 1 + (moving ? 1 : 0);
      for (int a0 = 0; a0 < na; a0 += 32) {
        const int a = a0 + lane;
        double x = 0.0, y = 0.0;
        int xg = 0, yg = 0;
        if (a < na) {
          if (first + a <= s1) { x = __ldg(&path[first + a].x); y = __ldg(&path[first + a].y); }
          else { const BeamLoc L = beam_loc(P, path, t_end, s1); x = L.x; y = L.y; }
          xg = (int)floor(rn_div(rn_sub(x, P.xmin), P.xres));
          yg = (int)floor(rn_div(rn_sub(y, P.ymin), P.yres));
        }
        const bool inside = !(xg < 0 || xg > P.nx - 1 || yg < 0 || yg > P.ny - 1);
        if (pass == 0) {
          unsigned todo = __ballot_sync(0xffffffffu, a < na && !inside);
          while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1;
            const double ax = __shfl_sync(0xffffffffu, x, src), ay = __shfl_sync(0xffffffffu, y, src);
            const int gx = __shfl_sync(0xffffffffu, xg, src), gy = __shfl_sync(0xffffffffu, yg, src);
            if (gx < 0) perimeter_edge(P, true, 0, ax, ay, B.r2, sink);
            if (gx > P.nx - 1) perimeter_edge(P, true, P.nx - 1, ax, ay, B.r2, sink);
            if (gy < 0) perimeter_edge(P, false, 0, ax, ay, B.r2, sink);
            if (gy > P.ny - 1) perimeter_edge(P, false, P.ny - 1, ax, ay, B.r2, sink);
          }
        } else {
          // eight anchors per round, four lanes each
          const unsigned in_m = __ballot_sync(0xffffffffu, a < na && inside);
          for (int g = 0; g < 32 && (in_m >> g) != 0u; g += 8) {
            const int src = g + (lane >> 2);
            const int gx = __shfl_sync(0xffffffffu, xg, src), gy = __shfl_sync(0xffffffffu, yg, src);
            bool has = false;
            int q = 0;
            if ((in_m >> src) & 1u) {
              const int i = gx + ((lane & 3) >> 1), j = gy + (lane & 1);
              if (!(i < 0 || i > P.nx - 1 || j < 0 || j > P.ny - 1)) { q = (int)pid(P, i, j, P.nz - 1); has = true; }
            }
            sink(has, q);
          }
        }
      }
    }
  }
}

// Appends the trace's points to a slot's seed list (warp-collective; n counts past the cap).
struct SeedSink {
  int* out;
  int cap;
  int n;
  __device__ void operator()(bool has, int q) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, has);
    if (has) {
      const int i = n + __popc(m & ((1u << lane) - 1u));
      if (i < cap) out[i] = q;
    }
    n += __popc(m);
  }
};

// ------------------------------------------------------------------ node windows
__global__ void __launch_bounds__(kGenThreads, 2) k_nodes_window(DevProblem P, NodeWindow w, int first, int n, int is_sol,
                                                              int* err) {
  __shared__ GenShared sh;
  extern __shared__ __align__(16) unsigned char gen_dyn[];    // GenComp of a compressing deck
  const int slot = first + blockIdx.x;
  const NodeBufView nb = slot_view(w, slot);
  gen_list_block(P, w.t[slot], is_sol != 0, nb, &w.count[slot], err, sh, P.compress ? (GenComp*)gen_dyn : nullptr);
  if (P.tracking != TH_TRACK_NONE && threadIdx.x < 32) {   // the step's beam-trace candidates
    SeedSink sink{w.seeds + (size_t)slot * w.seed_cap, w.seed_cap, 0};
    beam_trace(P, w.t[slot], sink);
    if (threadIdx.x == 0) {
      w.nseed[slot] = sink.n;
      if (sink.n > w.seed_cap) atomicOr(err, ERR_SEED_CAPACITY);
    }
  }
}

// Depth walk under a liquid surface point and the running depth maximum
// (src/Melt.cpp:271-357): walk down while liquid, else walk up solidifying.  The walk is
// sequential in the reference; here the layers it is likely to visit are evaluated four
// at a time ahead of it - the caller's first pass already holds D + 1 (down) and D (up) -
// and only the layers the walk reaches are committed.  T at a layer does not depend on the
// walk.
template <int PREC, bool RDF>
__device__ int depth_walk(const DevProblem& P, const TrackState& S, const StepCtx& X, int p, int D,
                          const EvalT& first_down, const EvalT& first_up, unsigned long long& pairs) {
  const int lane = threadIdx.x & 31;
  const int col = p / P.nz;
  const int top = col * P.nz + (P.nz - 1);            // layer d of the column is point top - d
  // FP64 runs walk one layer at a time: their passes are FP64-throughput bound, so layers
  // the walk may not reach are not evaluated ahead
  constexpr int NB = PREC == 0 ? 1 : 4;
  EvalT Tc[4], Tu[4];
  int cb = D + 1, cn = (PREC != 0 && D + 1 <= P.nz - 1) ? 1 : 0;   // down: cb..cb+cn-1
  int ub = D, un = (PREC != 0 && D >= 1) ? 1 : 0;                  // up: ub..ub-un+1
  Tc[0] = first_down; Tu[0] = first_up;
  int d = D;
  bool none_deeper = true;
  while (true) {
    ++d;
    if (d == P.nz) break;
    if (d >= cb + cn) {                               // next NB layers down
      int pts[NB];
      cn = 0;
#pragma unroll
      for (int q = 0; q < NB; ++q) {
        const bool ok = d + q <= P.nz - 1;
        pts[q] = ok ? top - (d + q) : p;
        cn += ok ? 1 : 0;
      }
      cb = d;
      EvalT tmp[NB];
      eval_Tn<PREC, NB>(P, S, X, pts, tmp);
#pragma unroll
      for (int q = 0; q < NB; ++q) Tc[q] = tmp[q];
    }
    EvalT T = pick4(Tc, d - cb);
    guard_T<PREC>(P, S, X, T, top - d);
    pairs += X.nn;
    if (lane == 0) set_T(S, top - d, T, X.k);
    if (!T.liquid) break;
    if (RDF && lane == 0) rdf_melt(S, X, top - d);
    none_deeper = false;
  }
  EvalT Tl4[4];                                       // the up layers' T at t - dt (below D)
  while (true) {
    --d;
    if (d == 0 || !none_deeper) break;
    if (!(d <= ub && d > ub - un)) {                  // next NB layers up, at t and at t - dt
      int pts[NB];
      un = 0;
#pragma unroll
      for (int q = 0; q < NB; ++q) {
        const bool ok = d - q >= 1;
        pts[q] = ok ? top - (d - q) : p;
        un += ok ? 1 : 0;
      }
      ub = d;
      EvalT tmp[NB], tmpl[NB];
      eval_Tn<PREC, NB>(P, S, X, pts, tmp);
      // T at t - dt is needed only below D (the layer at D has it stored)
      if (d != D) {
        const long long c0 = clock64();
        warp_T_n<PREC, NB>(P, S, X.ax, X.nbl, X.nnl, pts, X.stl, tmpl);
        X.ev_c += clock64() - c0;
        X.ev_n += 1;
        X.ev_nodes += X.nnl;
      }
#pragma unroll
      for (int q = 0; q < NB; ++q) { Tu[q] = tmp[q]; Tl4[q] = tmpl[q]; }
    }
    const int q = top - d;
    const double Told = ldcg_d(S.T + q);
    EvalT T = pick4(Tu, ub - d);
    guard_T<PREC>(P, S, X, T, q);
    pairs += X.nn;
    if (lane == 0) set_T(S, q, T, X.k);
    if (!T.liquid) {
      double Tl = Told;                                   // T of the previous step
      if (d != D) { Tl = pick4(Tl4, ub - d).T; pairs += X.nnl; }
      if (lane == 0) push_rec<RDF ? TM_SURFACE_RDF : TM_SURFACE>(S, X, q, T.T, Tl);
    } else {
      if (RDF && lane == 0) rdf_melt(S, X, q);
      break;
    }
  }
  if (d == P.nz) --d;
  if (lane == 0) {
    S.depths[col] = d;
    if (S.depth) {
      double dep;
      if (d == P.nz - 1) dep = d;
      else {
        const double Tl = t_decode(S, P, ldcg_d(S.T + col * P.nz + (P.nz - 1 - d)));
        const double Ts = t_decode(S, P, ldcg_d(S.T + col * P.nz + (P.nz - 1 - (d + 1))));
        dep = rn_add((double)d, rn_div(rn_sub(P.TL, Tl), rn_sub(Ts, Tl)));
      }
      if (dep > S.depth_max[col]) {
        S.depth_max[col] = dep;
        for (int dd = d; dd >= 0; --dd) S.depth[col * P.nz + (P.nz - 1 - dd)] = dep;
      }
    }
  }
  return d;
}

// Stork's depth walk (src/Run.cpp:909-956): down while liquid, else up until liquid, on T at
// t alone; only the column's depth is kept.  A walk that ends on the bottom layer keeps the
// layer above it (the reference's bottom rule).  Layers are evaluated ahead as in
// depth_walk.
template <int PREC>
__device__ int stork_walk(const DevProblem& P, const TrackState& S, const StepCtx& X, int p, int D,
                          const EvalT& first_down, const EvalT& first_up, unsigned long long& pairs) {
  const int lane = threadIdx.x & 31;
  const int col = p / P.nz;
  const int top = col * P.nz + (P.nz - 1);
  constexpr int NB = PREC == 0 ? 1 : 4;
  EvalT Tc[4], Tu[4];
  int cb = D + 1, cn = (PREC != 0 && D + 1 <= P.nz - 1) ? 1 : 0;
  int ub = D, un = (PREC != 0 && D >= 1) ? 1 : 0;
  Tc[0] = first_down; Tu[0] = first_up;
  int d = D;
  bool none_deeper = true;
  while (true) {
    ++d;
    if (d == P.nz) break;
    if (d >= cb + cn) {
      int pts[NB];
      cn = 0;
#pragma unroll
      for (int q = 0; q < NB; ++q) {
        const bool ok = d + q <= P.nz - 1;
        pts[q] = ok ? top - (d + q) : p;
        cn += ok ? 1 : 0;
      }
      cb = d;
      EvalT tmp[NB];
      eval_Tn<PREC, NB>(P, S, X, pts, tmp);
#pragma unroll
      for (int q = 0; q < NB; ++q) Tc[q] = tmp[q];
    }
    EvalT T = pick4(Tc, d - cb);
    guard_T<PREC>(P, S, X, T, top - d);
    pairs += X.nn;
    if (!T.liquid) break;
    none_deeper = false;
  }
  while (true) {
    --d;
    if (d == 0 || !none_deeper) break;
    if (!(d <= ub && d > ub - un)) {
      int pts[NB];
      un = 0;
#pragma unroll
      for (int q = 0; q < NB; ++q) {
        const bool ok = d - q >= 1;
        pts[q] = ok ? top - (d - q) : p;
        un += ok ? 1 : 0;
      }
      ub = d;
      EvalT tmp[NB];
      eval_Tn<PREC, NB>(P, S, X, pts, tmp);
#pragma unroll
      for (int q = 0; q < NB; ++q) Tu[q] = tmp[q];
    }
    EvalT T = pick4(Tu, ub - d);
    guard_T<PREC>(P, S, X, T, top - d);
    pairs += X.nn;
    if (T.liquid) break;
  }
  if (d == P.nz - 1) --d;
  if (lane == 0) S.depths[col] = d;
  return d;
}

// One work item; returns the number of child items it published (already counted).
// A beam-trace candidate arrives with its claim still in flight (the lane-0 result of the
// atomic, `got`): the point is evaluated meanwhile and the item stops before any effect if
// another item took the point.
// A re-test brings its column's depth from the liquid list (Dk); other items read it.
// Stork re-tests (src/Run.cpp:796-830) expand only when still liquid, and one that cooled
// only resets its column's depth.
template <int PREC, int TM>
__device__ int run_item(const DevProblem& P, const TrackState& S, const StepCtx& X, int type, int p, int aux,
                        int Dk, bool seed, bool got, unsigned long long& pairs, Kept& kept) {
  constexpr bool SURF = TM != TM_VOLUME;
  constexpr bool STORK = TM == TM_STORK;
  constexpr bool RDF = TM == TM_SURFACE_RDF;
  constexpr bool RETEST_EXPANDS = SURF && !STORK;     // Surface: test_pts = last_liq_pts
  const int lane = threadIdx.x & 31;
  int nchild = 0;
  const double Told = ldcg_d(S.T + p);
  if (type == IT_COLUMN) {                 // a layer under a surface point that solidified
    EvalT T = eval_T<PREC>(P, S, X, X.nb, X.nn, p, X.st);
    guard_T<PREC>(P, S, X, T, p);
    pairs += X.nn;
    if (lane == 0) set_T(S, p, T, X.k);
    double Tl = Told;
    if (aux) { Tl = eval_T<PREC>(P, S, X, X.nbl, X.nnl, p, X.stl).T; pairs += X.nnl; }
    if (lane == 0) push_rec<TM>(S, X, p, T.T, Tl);
    if (RDF && lane == 0 && T.liquid) rdf_melt(S, X, p);   // solidified while still liquid
    return 0;
  }
  // Surface re-tests expand whatever their temperature (src/Run.cpp:655): the claims are
  // issued first and run while this point is evaluated; the claimed neighbours are
  // published after the pass.
  Claims rc{0, 0, 0xffffffffu};
  if (RETEST_EXPANDS && type == IT_RETEST) rc = claim_neighbours<SURF>(P, S, X, p);
  EvalT T3[3];
  int D = 0;
  if (SURF && PREC != 0) {                 // the point and the layers its depth walk starts with
    const int col = p / P.nz, top = col * P.nz + (P.nz - 1);
    D = type == IT_RETEST ? Dk : (seed ? ldcg_i(S.depths + col) : aux);
    const int down = D + 1 <= P.nz - 1 ? top - (D + 1) : p;
    if (D >= 1) {
      const int pts[3] = {p, down, top - D};
      eval_Tn<PREC, 3>(P, S, X, pts, T3);
    } else {
      const int pts[2] = {p, down};
      EvalT T2[2];
      eval_Tn<PREC, 2>(P, S, X, pts, T2);
      T3[0] = T2[0]; T3[1] = T2[1]; T3[2] = T2[1];
    }
  } else {
    if (SURF) D = type == IT_RETEST ? Dk : (seed ? ldcg_i(S.depths + p / P.nz) : aux);
    T3[0] = eval_T<PREC>(P, S, X, X.nb, X.nn, p, X.st);
  }
  if (RETEST_EXPANDS && type == IT_RETEST) emit_claimed<SURF>(S, X, rc, nchild, nullptr);
  if (seed && !__shfl_sync(0xffffffffu, got, 0)) return 0;
  EvalT T = T3[0];
  guard_T<PREC>(P, S, X, T, p);
  pairs += X.nn;
  if (lane == 0) set_T(S, p, T, X.k);
  if (T.liquid) {
    int slot = 0;
    if (lane == 0) slot = atomicAdd(X.lo_n, 1);
    if (RDF && lane == 0) rdf_melt(S, X, p);
    // Volume expands the liquid points; Surface the liquid visits (re-tests did above)
    // Volume items keep one claimed neighbour to run next in the same warp; Surface items
    // publish all of them (a kept child would wait for the rest of a long re-test or depth
    // walk, longer than the queue takes to hand it to another warp)
    if (!(RETEST_EXPANDS && type == IT_RETEST)) expand<SURF>(P, S, X, p, nchild, SURF ? nullptr : &kept);
    // the depth walk under a liquid surface point needs nothing else from this step
    int Dn = 0;
    if (STORK) Dn = stork_walk<PREC>(P, S, X, p, D, T3[1], T3[2], pairs);
    else if (SURF) Dn = depth_walk<PREC, RDF>(P, S, X, p, D, T3[1], T3[2], pairs);
    if (lane == 0) push_liquid(S, X, slot, p, Dn);
    if (STORK && lane == 0) log_liquid(S, X, slot, p, Dn);
  } else if (STORK) {
    if (type == IT_RETEST && lane == 0) S.depths[p / P.nz] = 0;
  } else if (type == IT_RETEST) {          // cooled below T_L since the last step
    if (lane == 0) push_rec<TM>(S, X, p, T.T, Told);
    if (SURF) {
      const int col = p / P.nz;
      for (int d0 = 1; d0 <= D; d0 += 32) {
        const int d = d0 + lane;
        emit<SURF>(S, X, d <= D, IT_COLUMN, col * P.nz + (P.nz - 1 - d), d != D, nchild);
      }
      if (lane == 0) S.depths[col] = 0;
    }
  }
  return nchild;
}

// Volume items come in batches: the previous step's liquid points are re-tested kVolChunk at
// a time, and an item evaluates the neighbours it claims itself, kVolBatch to a pass
// (warp_T_gen), publishing only those found liquid, as IT_EXPAND items (a liquid point whose
// neighbours are still to be claimed).  The sets of claims, evaluations and decisions are
// the one-point-per-item loop's (src/Melt.cpp:185-269): a claim is the same atomic, and a
// point's sum is bit for bit the same in a batch.
constexpr int kVolChunk = 3;     // re-tests per initial item
constexpr int kVolBatch = 3;     // points per evaluation pass (3 ran 2 % faster than 4)
constexpr int kVolCand = 18 * kVolChunk;   // most neighbours one item can claim
static_assert(kVolChunk <= kVolBatch, "a chunk of re-tests is one pass");

// One pass over the first n points of a batch (a pass of 1, 2 or kVolBatch points; pts
// padded by repeating a point).
template <int PREC>
__device__ __forceinline__ void vol_pass(const DevProblem& P, const TrackState& S, const StepCtx& X,
                                         const int (&pts)[kVolBatch], int n, EvalT (&T)[kVolBatch]) {
  static_assert(kVolBatch >= 2 && kVolBatch <= 4, "passes of 1, 2 or kVolBatch points");
  const long long c0 = clock64();
  if (n == 1) {
    const int p1[1] = {pts[0]};
    EvalT t1[1];
    warp_T_gen<PREC, 1>(P, S, X.ax, X.nb, X.nn, p1, X.st, t1);
    T[0] = t1[0];
  } else if (kVolBatch == 2 || n == 2) {
    const int p2[2] = {pts[0], pts[1]};
    EvalT t2[2];
    warp_T_gen<PREC, 2>(P, S, X.ax, X.nb, X.nn, p2, X.st, t2);
    T[0] = t2[0]; T[1] = t2[1];
  } else {
    if constexpr (kVolBatch > 2) warp_T_gen<PREC, kVolBatch>(P, S, X.ax, X.nb, X.nn, pts, X.st, T);
  }
  X.ev_c += clock64() - c0;
  X.ev_n += 1;
  X.ev_nodes += X.nn;
}

// Stores the T of the batch's first n points and returns which are liquid (bit q: pts[q]).
template <int PREC>
__device__ __forceinline__ unsigned vol_commit(const DevProblem& P, const TrackState& S, const StepCtx& X,
                                               const int (&pts)[kVolBatch], int n, EvalT (&T)[kVolBatch],
                                               unsigned long long& pairs) {
  const int lane = threadIdx.x & 31;
  unsigned liq = 0;
#pragma unroll
  for (int q = 0; q < kVolBatch; ++q) {
    if (q >= n) break;
    guard_T<PREC>(P, S, X, T[q], pts[q]);
    pairs += X.nn;
    if (lane == 0) set_T(S, pts[q], T[q], X.k);
    if (T[q].liquid) liq |= 1u << q;
  }
  return liq;
}

// Claims the neighbours of the nE liquid points E (the same 3x3x{k-1, k} claims as
// expand), evaluates the newly claimed ones in batches, adds the liquid ones to the next
// step's list and publishes them as IT_EXPAND items (keeping one for this warp to run
// next).  `cand` is the warp's slice of shared memory (kVolCand entries).
template <int PREC>
__device__ void vol_expand(const DevProblem& P, const TrackState& S, const StepCtx& X, const int (&E)[kVolChunk],
                           int nE, int* cand, int& nchild, unsigned long long& pairs, Kept& kept) {
  const int lane = threadIdx.x & 31;
  Claims c[kVolChunk];
#pragma unroll
  for (int i = 0; i < kVolChunk; ++i)              // every claim in flight before any result is used
    if (i < nE) c[i] = claim_neighbours<false>(P, S, X, E[i]);
  int n = 0;
#pragma unroll
  for (int i = 0; i < kVolChunk; ++i) {
    if (i >= nE) break;
    const bool got = c[i].old < X.stamp;
    const unsigned m = __ballot_sync(0xffffffffu, got);
    if (got) cand[n + __popc(m & ((1u << lane) - 1u))] = c[i].q;
    n += __popc(m);
  }
  __syncwarp();
  for (int b = 0; b < n; b += kVolBatch) {
    const int nb = min(kVolBatch, n - b);
    int pts[kVolBatch];
#pragma unroll
    for (int q = 0; q < kVolBatch; ++q) pts[q] = cand[b + min(q, nb - 1)];
    EvalT T[kVolBatch];
    vol_pass<PREC>(P, S, X, pts, nb, T);
    const unsigned liq = vol_commit<PREC>(P, S, X, pts, nb, T, pairs);
    int slot = 0;
    if (lane == 0 && liq) slot = atomicAdd(X.lo_n, __popc(liq));
    // lane q < nb carries point q; the liquid ones join the list and the queue
    int mine = pts[0];
#pragma unroll
    for (int q = 1; q < kVolBatch; ++q) if (lane == q) mine = pts[q];
    const bool is_liq = lane < nb && ((liq >> lane) & 1u);
    slot = __shfl_sync(0xffffffffu, slot, 0) + __popc(liq & ((1u << lane) - 1u));
    if (is_liq) push_liquid(S, X, slot, mine, 0);
    emit<false>(S, X, is_liq, IT_EXPAND, mine, 0, nchild, &kept);
    __syncwarp();
  }
}

// One Volume item (see kVolChunk): a chunk of `units` re-tests starting at list entry p
// (IT_RETEST), a beam-trace candidate (IT_VISIT), or a liquid point to expand (IT_EXPAND).
template <int PREC>
__device__ int run_item_vol(const DevProblem& P, const TrackState& S, const StepCtx& X, int type, int p, int units,
                            bool seed, bool got, int* cand, unsigned long long& pairs, Kept& kept) {
  const int lane = threadIdx.x & 31;
  int nchild = 0;
  int E[kVolChunk];
  int nE = 0;
  if (type == IT_RETEST) {
    int pts[kVolBatch];
    double Told[kVolBatch];
#pragma unroll
    for (int q = 0; q < kVolBatch; ++q) {
      pts[q] = __ldcg(X.L + p + min(q, units - 1)).x;
      Told[q] = ldcg_d(S.T + pts[q]);
    }
    EvalT T[kVolBatch];
    vol_pass<PREC>(P, S, X, pts, units, T);
    const unsigned liq = vol_commit<PREC>(P, S, X, pts, units, T, pairs);
    int slot = 0;
    if (lane == 0 && liq) slot = atomicAdd(X.lo_n, __popc(liq));
#pragma unroll
    for (int q = 0; q < kVolBatch; ++q) {
      if (q >= units) break;
      if ((liq >> q) & 1u) {
        if (lane == 0) push_liquid(S, X, slot + __popc(liq & ((1u << q) - 1u)), pts[q], 0);
        E[nE++] = pts[q];
      } else if (lane == 0) {
        push_rec<TM_VOLUME>(S, X, pts[q], T[q].T, Told[q]);    // cooled below T_L since the last step
      }
    }
  } else if (type == IT_VISIT) {
    int pts[kVolBatch];
#pragma unroll
    for (int q = 0; q < kVolBatch; ++q) pts[q] = p;
    EvalT T[kVolBatch];
    vol_pass<PREC>(P, S, X, pts, 1, T);              // the claim's result arrives meanwhile
    if (seed && !__shfl_sync(0xffffffffu, got, 0)) return 0;   // another item took the point
    const unsigned liq = vol_commit<PREC>(P, S, X, pts, 1, T, pairs);
    if (liq) {
      int slot = 0;
      if (lane == 0) slot = atomicAdd(X.lo_n, 1);
      if (lane == 0) push_liquid(S, X, slot, p, 0);
      E[nE++] = p;
    }
  } else {
    E[nE++] = p;
  }
  if (nE) vol_expand<PREC>(P, S, X, E, nE, cand, nchild, pairs, kept);
  return nchild;
}

// ------------------------------------------------------------------ the tracking loop
// Warps per block, one block per SM: Surface steps are short chains of ~500 items (latency-
// bound; more waiting warps only add polls), Volume steps have ~1e5 items (throughput-
// bound: twelve warps share one staged copy of the lists).
template <bool SURF>
__host__ __device__ constexpr int track_threads() { return SURF ? 128 : 384; }
// The thread bound the kernel is compiled for.  Volume: 512 threads hold it to 128 registers
// (a few hundred bytes of spills), so that each of the SM's four register partitions
// (16,384 registers) takes three tracking warps and one warp of a 128-thread, 128-register
// bulk-solidification block of the other stream.  Eight warps at 168 registers ran the run
// 9 % slower (4.74 against 4.33 s), nine at 168 left a partition no room for the
// solidification warp (its windows waited for the tracking launches: 5.24 s), ten at 128
// took 4.82 s, sixteen at 96 4.57 s; at its unconstrained 230 registers the solidification
// of a window waited for the tracking launch and ran after it.
template <bool SURF>
constexpr int track_bound() { return SURF ? 128 : 512; }
// The first 48 bytes of a step's QueueCounters (head, depth, lvl_start, lvl_end) into
// shared memory, bypassing L1 (the counters are updated by atomics in L2).
__device__ __forceinline__ void copy_step_prof(const QueueCounters* q, unsigned* dst) {
  for (int c = 0; c < 3; ++c) cp_async16(dst + 4 * c, (const unsigned*)q + 4 * c);
  cp_async_commit();
}
__device__ __forceinline__ void add_step_prof(const unsigned* q, unsigned long long* acc) {
  acc[0] += q[1];                                   // depth
  for (int l = 0; l < 4; ++l) { acc[1 + l] += q[2 + l]; acc[5 + l] += q[6 + l]; }
}

// FP32 tracking keeps the grid's axis table (8 bytes per axis point) in shared memory
// behind the staged lists when the axes have at most kAxisSmem points in all.
constexpr int kAxisSmem = 2048;
template <int PREC>
__host__ __device__ __forceinline__ bool axis_in_smem(const DevProblem& P) {
  return PREC != 0 && P.nx + P.ny + P.nz <= kAxisSmem;
}

// One launch runs steps [k_begin, k_end) of a Volume or Surface loop (src/Run.cpp:469-709).
// Each step is a single phase: the previous step's liquid points are re-tested, the beam
// trace seeds the new ones, and every claimed point, column and depth walk becomes a work
// item that any warp may take; the step word (entered blocks, published and completed
// items) tells when the step has no work left, and the step's end is published as one word
// that the waiting warps poll (no grid barrier).
//
// spin_limit bounds every wait (kSpinLimit unless a test lowers it); hold (a test knob, 0
// otherwise) counts items into every step that are never dealt, so no step can end and the
// waits run out: the path of a lost item.
template <int PREC, int TM>
__global__ void __launch_bounds__(track_bound<TM != TM_VOLUME>(), 1) k_track(DevProblem P, TrackState S, NodeWindow W,
                                                                        int k_begin, int k_end, int high_water,
                                                                        int stage_cap, long long spin_limit, int hold) {
  constexpr bool SURF = TM != TM_VOLUME;
  constexpr bool VOL = TM == TM_VOLUME;
  // Volume: each warp's neighbours claimed by one item, before they are evaluated
  __shared__ int s_cand[VOL ? track_threads<false>() / 32 : 1][VOL ? kVolCand : 1];
  const int tid_w = VOL ? (int)(threadIdx.x >> 5) : 0;
  extern __shared__ __align__(16) unsigned char stage_mem[];
  __shared__ BlockBuf bbuf;
  const int lane = threadIdx.x & 31;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_warps = (gridDim.x * blockDim.x) >> 5;
  TrackCounters* C = S.C;
  unsigned long long pairs = 0;
  const size_t buf_bytes = (size_t)stage_cap * staged_bytes_per_node<PREC>();
  __shared__ int s_flush[2];
  if (threadIdx.x == 0) bbuf.nrec = 0;
  // Three staged lists rotate by step: k % 3 holds step k's, (k - 1) % 3 the previous
  // step's (for T at t - dt), (k + 1) % 3 receives the next step's while step k runs.
  auto buf_of = [&](int kk) { return stage_mem + (size_t)(((kk % 3) + 3) % 3) * buf_bytes; };
  if (k_begin < k_end) {
    const int slot = k_begin - W.base + 1;
    stage_issue<PREC>(slot_view(W, slot), min(W.count[slot], stage_cap), buf_of(k_begin), stage_cap);
    if (k_begin > 0) stage_issue<PREC>(slot_view(W, slot - 1), min(W.count[slot - 1], stage_cap), buf_of(k_begin - 1),
                                       stage_cap);
  }
  // the axis table after the three lists, when it fits
  const float2* ax = S.axis;
  if (axis_in_smem<PREC>(P)) {
    float2* sax = (float2*)(stage_mem + 3 * buf_bytes);
    for (int i = threadIdx.x; i < P.nx + P.ny + P.nz; i += blockDim.x) sax[i] = __ldg(S.axis + i);
    ax = sax;
  }
  cp_async_wait_all();
  __syncthreads();
  unsigned long long t_work = 0, n_items = 0, c_items = 0, c_wait = 0;
  unsigned long long ev_n = 0, ev_c = 0, ev_nodes = 0;
  // block 0's per-step profile (chain depth, latest item start / end per depth): each
  // step's counters are copied asynchronously at its end and folded in a step later
  __shared__ __align__(16) unsigned s_qprof[2][12];
  __shared__ unsigned long long s_acc[9];
  bool prof_pend = false;
  if (threadIdx.x == 0)
    for (int i = 0; i < 9; ++i) s_acc[i] = 0ull;
  // step k's live-list length and this warp's first re-test entry, read when step k - 1
  // ended (for the first step, from memory)
  int nL_next = k_begin < k_end ? ldcg_i(&C->liq_n[k_begin % 3]) : 0;
  // Stork: the launch's log starts with the liquid list of step k_begin - 1 (list 0); the
  // list each step fills follows the one before it
  int log_pos = nL_next;
  if (TM == TM_STORK && blockIdx.x == 0 && k_begin < k_end) {
    const int2* L0 = S.liq[k_begin % 3];
    for (int i = threadIdx.x; i < nL_next && i < S.rlog_cap; i += blockDim.x) S.rlog[i] = __ldcg(L0 + i);
    if (threadIdx.x == 0) { S.rlog_off[0] = 0; S.rlog_off[1] = nL_next; }
  }
  int2 first_next = make_int2(0, 0);
  if (k_begin < k_end && (tid >> 5) < S.list_cap) first_next = __ldcg(S.liq[k_begin % 3] + (tid >> 5));
  // the window's per-step scalars, read one step ahead
  double t_next = 0.0;
  int cnt_next = 0, cntl_next = 0, nseed_next = 0;
  if (k_begin < k_end) {
    const int slot = k_begin - W.base + 1;
    t_next = W.t[slot]; cnt_next = W.count[slot]; cntl_next = W.count[slot - 1]; nseed_next = W.nseed[slot];
  }
  // Surface forms: this block's last flush took the record buffer past its high-water mark
  // (the block's next step entry asks for the launch to end after that step)
  bool stop_vote = false;
  int k = k_begin;
  for (; k < k_end; ++k) {
    StepCtx X;
    X.ev_n = 0;
    X.ev_c = 0;
    X.ev_nodes = 0;
    const int slot = k - W.base + 1;
    const double t_k = t_next;
    const int cnt_k = cnt_next, cntl_k = cntl_next, nseed_k = nseed_next;
    if (k + 1 < k_end) {
      t_next = W.t[slot + 1]; cnt_next = W.count[slot + 1]; cntl_next = cnt_k; nseed_next = W.nseed[slot + 1];
    }
    const unsigned long long g0 = globaltimer();
    int max_depth = 0;
    const int b0 = k % 3, b1 = (k + 1) % 3;
    X.qc = &C->q[b0];
    X.stamp = (unsigned)k + 1u;
    X.nL = nL_next;
    const int2 first_entry = first_next;
    // the beam trace runs for k > 0 while t < end + dt (src/Run.cpp:661)
    X.t = t_k;
    const bool seeds = k > 0 && X.t < P.end_time + P.dt;
    const int n_seed = seeds ? min(nseed_k, W.seed_cap) : 0;
    const int* seed = W.seeds + (size_t)slot * W.seed_cap;
    X.n_init = X.nL + n_seed;
    // the next step's list is copied while this step runs, issued by each warp when it
    // first runs out of initial items
    bool staged = !(k + 1 < k_end);
    X.bb = &bbuf;
    X.st.base = buf_of(k);
    X.st.cap = stage_cap;
    X.st.n_sm = min(cnt_k, stage_cap);
    X.stl.base = buf_of(k - 1);
    X.stl.cap = stage_cap;
    X.stl.n_sm = k == 0 ? 0 : min(cntl_k, stage_cap);
    X.k = k;
    X.nb = slot_ref(W, slot);
    X.nbl = slot_ref(W, slot - 1);
    X.nn = min(cnt_k, W.slot_cap);
    X.nnl = (k == 0) ? 0 : min(cntl_k, W.slot_cap);
    X.L = S.liq[b0];
    X.Lo = S.liq[b1];
    X.lo_n = &C->liq_n[b1];
    X.ax = ax;
    X.log_out = log_pos;
    X.log_j = k - k_begin + 1;
    X.hw = high_water;
    X.liq = 0;
    // this block enters the step (thread 0; Surface forms: once its warp has run out of
    // initial items - the entry waits for the clears before it, and the step cannot end
    // before those items anyway)
    unsigned long long arrival = 0;
    bool arrival_pending = threadIdx.x == 0;
    if (VOL && arrival_pending) arrival = atomicAdd(&X.qc->state, StepWord<false>::kArrive);
    // The work loop.  The step's initial items - re-tests of the previous liquid points,
    // then the beam trace's candidates - are dealt to the warps in order (warp w takes
    // w, w + warps, ...), so they all start at once; items published during the step are
    // taken with tickets from the queue.  The step is over when every block has entered
    // it and every item has completed; whoever's update of the step word makes that true
    // publishes the step-end word, which the waiting warps see (Volume: after resetting
    // the counters the next steps use and reading the next list's length and the record
    // count; Surface forms: at once, the step word holding the list's length and any stop
    // request, the counters cleared by the blocks as they entered the step).  No grid
    // barrier separates steps.  (Surface forms whose waiting warps read the end from the
    // step word itself, with no step-end word, took 6 % longer: ~600 warps polling the
    // line that the step's atomics update.)
    // Volume deals the re-tests kVolChunk to an item; an item completes as many initial
    // entries as it took (one, or its chunk's re-tests).  Volume warps take the initial items
    // from a counter (a warp runs about ten a step, of uneven cost); Surface and Stork deal
    // them by warp, so that they all start at once without a round trip.
    const int n_rt = VOL ? (X.nL + kVolChunk - 1) / kVolChunk : X.nL;
    const int n_units = n_rt + n_seed;
    int next_init = VOL ? 0 : tid >> 5;
    long long idle = 0;
    unsigned long long fin_seen = 0xffffffffull;   // the step-end word this warp saw
    while (true) {
      const long long c0 = clock64();
      int type, p = 0, aux = 0, Dk = 0, units = 1;
      bool is_seed = false, got = false;
      int t = -1;
      if (next_init < n_units) {
        if (VOL) {
          unsigned u = 0;
          if (lane == 0) u = atomicAdd(&X.qc->init_head, 1u);
          u = __shfl_sync(0xffffffffu, u, 0);
          if ((int)u < n_units) t = (int)u; else next_init = n_units;   // none left this step
        } else {
          t = next_init;
          next_init += n_warps;
        }
      }
      if (t >= 0) {
        X.depth = 0;
        if (t < n_rt) {
          type = IT_RETEST;
          if (VOL) {                        // entries [p, p + units) of the list
            p = t * kVolChunk;
            units = min(kVolChunk, X.nL - p);
          } else {
            const int2 e = (t == (tid >> 5)) ? first_entry : __ldcg(X.L + t);
            p = e.x;
            Dk = e.y;
          }
        } else {                            // a trace candidate: visited if this claim takes it
          type = IT_VISIT;
          p = __ldg(seed + (t - n_rt));
          is_seed = true;
          if (lane == 0) got = claim(S, p, X.stamp);
        }
      } else {
        if (!staged) {
          stage_issue<PREC>(slot_view(W, slot + 1), min(cnt_next, stage_cap), buf_of(k + 1), stage_cap);
          staged = true;
        }
        if (arrival_pending) {              // this block's entry, checked once its result is back
          arrival_pending = false;
          if constexpr (SURF) {
            clear_counters(C, k);
            if (stop_vote) red_or(&X.qc->state, kSurfStop);
            stop_vote = false;
            arrival = atom_add_release(&X.qc->state, StepWord<true>::kArrive);   // after the clears and the vote
          }
          const unsigned long long v = arrival + StepWord<SURF>::kArrive;
          if constexpr (SURF) {
            if (StepWord<true>::over(v, X.n_init + hold, gridDim.x)) surface_finish<TM>(P, S, X, v);
          } else {
            if (StepWord<false>::over(v, X.n_init + hold, gridDim.x)) finish_step(P, S, X, k, v, high_water);
          }
        }
        unsigned ticket = 0;
        if (lane == 0) ticket = atomicAdd(&X.qc->head, 1u);
        ticket = __shfl_sync(0xffffffffu, ticket, 0);
        const unsigned j = ticket;
        bool ready = false, finished = false;
        unsigned long long fin = 0;
        unsigned backoff = 8;
        ulonglong2 it = make_ulonglong2(0ull, 0ull);
        while (true) {
          // one round trip for both: lane 0 reads the ticket's slot, lane 1 the step-end word
          // (read one after the other they took two: Surface 1 %, Volume 2.7 % slower)
          if (lane == 0) {
            if (j < (unsigned)S.queue_cap) it = ld_relaxed_v2(S.queue + j);
            ready = (unsigned)(it.x >> 32) == X.stamp && (unsigned)(it.y >> 32) == X.stamp;
          } else if (lane == 1) {
            fin = ld_acquire_u64(&C->fin);
            finished = (unsigned)fin >= X.stamp;
          }
          ready = __shfl_sync(0xffffffffu, ready, 0);
          finished = !ready && __shfl_sync(0xffffffffu, finished, 1);
          fin = ((unsigned long long)__shfl_sync(0xffffffffu, (unsigned)(fin >> 32), 1) << 32) |
                __shfl_sync(0xffffffffu, (unsigned)fin, 1);
          if (ready || finished) break;
          backoff = backoff < 64 ? backoff * 2 : 64;
          if (++idle > spin_limit) {
            if (lane == 0) {
              if (atomicOr(S.err, ERR_BARRIER) == 0) {        // first waiter to give up records its view
                using SW = StepWord<SURF>;
                const unsigned long long st = ld_relaxed_u64(&X.qc->state);
                int* g = S.C->diag;
                g[0] = 1; g[1] = k; g[2] = (int)j; g[3] = X.n_init;
                g[4] = (int)*(volatile unsigned*)&X.qc->head; g[5] = (int)SW::entered(st);
                g[6] = (int)SW::published(st); g[7] = (int)SW::completed(st);
              }
              st_release_u64(&C->fin, 0xffffffffull);       // let every warp leave
            }
            fin = 0xffffffffull;
            finished = true;
            break;
          }
          __nanosleep(backoff);
        }
        if (!ready) {
          fin_seen = ((unsigned long long)__shfl_sync(0xffffffffu, (unsigned)(fin >> 32), 0) << 32) |
                     __shfl_sync(0xffffffffu, (unsigned)fin, 0);
          c_wait += clock64() - c0;
          break;
        }
        const unsigned w0 = __shfl_sync(0xffffffffu, (unsigned)it.x, 0);
        const unsigned w1 = __shfl_sync(0xffffffffu, (unsigned)it.y, 0);
        p = (int)w0;
        type = w1 & 0xff;
        X.depth = (w1 >> 8) & 0xff;
        aux = (int)(w1 >> 16);
      }
      const long long c1 = clock64();
      c_wait += c1 - c0;
      if (X.depth > max_depth) {
        max_depth = X.depth;
        if (lane == 0) atomicMax(&X.qc->depth, (unsigned)max_depth);
      }
      unsigned long long g_item = globaltimer();
      Kept kept{0, 0, false};
      X.liq = 0;
      while (true) {
        if constexpr (VOL) run_item_vol<PREC>(P, S, X, type, p, units, is_seed, got, s_cand[tid_w], pairs, kept);
        else run_item<PREC, TM>(P, S, X, type, p, aux, Dk, is_seed, got, pairs, kept);
        if (lane == 0) {
          const int l = min(X.depth, 3);
          atomicMax(&X.qc->lvl_start[l], (unsigned)(g_item - g0));
          atomicMax(&X.qc->lvl_end[l], (unsigned)(globaltimer() - g0));
        }
        if (!kept.valid) break;
        // the kept child runs next; the item completes once its chain of kept children ends
        type = VOL ? IT_EXPAND : IT_VISIT; p = kept.p; aux = kept.aux; Dk = 0; is_seed = false; got = false;
        kept.valid = false;
        ++X.depth;
        if (X.depth > max_depth) {
          max_depth = X.depth;
          if (lane == 0) atomicMax(&X.qc->depth, (unsigned)max_depth);
        }
        ++n_items;
        g_item = globaltimer();
      }
      if (lane == 0) {                                           // completed, after the item's writes
        if constexpr (SURF) {
          const unsigned long long add = (unsigned long long)units | ((unsigned long long)X.liq << kSurfLiq);
          const unsigned long long v = atom_add_release(&X.qc->state, add) + add;
          if (StepWord<true>::over(v, X.n_init + hold, gridDim.x)) surface_finish<TM>(P, S, X, v);
        } else {
          const unsigned long long st = atom_add_release(&X.qc->state, (unsigned long long)units);
          if (StepWord<false>::over(st + units, X.n_init + hold, gridDim.x))
            finish_step(P, S, X, k, st + units, high_water);
        }
      }
      ++n_items;
      c_items += clock64() - c1;
    }
    t_work += globaltimer() - g0;
    ev_n += X.ev_n;
    ev_c += X.ev_c;
    ev_nodes += X.ev_nodes;
    // The step is over.  The word that ended this warp's wait carries the next step's
    // live-list length and the run's verdict, so every warp of the block takes the same
    // decisions without another load; the block barrier also completes the next list's
    // copies (and block 0's copy of the last step's profile counters).
    const bool aborted = (unsigned)fin_seen == 0xffffffffu;
    const unsigned verdict = (unsigned)(fin_seen >> 32) & 3u;
    nL_next = (int)(fin_seen >> 34);
    log_pos += nL_next;
    if (!VOL && !aborted && (tid >> 5) < S.list_cap) first_next = __ldcg(X.Lo + (tid >> 5));
    cp_async_wait_all();
    if (threadIdx.x == 0) s_flush[k & 1] = bbuf.nrec >= kBlkRec / 2;
    if (__syncthreads_or(aborted)) break;
    if (tid == 0) {                           // profile: fold the previous step's copy, copy this one's
      if (prof_pend) add_step_prof(s_qprof[(k - 1) & 1], s_acc);
      copy_step_prof(X.qc, s_qprof[k & 1]);
      prof_pend = true;
    }
    if (verdict) { ++k; break; }
    if (s_flush[k & 1]) {
      const int n_rec = flush_block(S, &bbuf, S.rec_n);
      stop_vote = SURF && n_rec > high_water;
    }
  }
  cp_async_wait_all();
  if (tid == 0 && prof_pend) add_step_prof(s_qprof[(k - 1) & 1], s_acc);
  flush_block(S, &bbuf, S.rec_n);
  if (lane == 0 && pairs) atomicAdd(S.pairs, pairs);
  if (lane == 0) {
    atomicAdd(&C->prof[2], n_items);
    atomicAdd(&C->prof[3], c_items);
    atomicAdd(&C->prof[4], c_wait);
    atomicAdd(&C->prof[7], ev_n);
    atomicAdd(&C->prof[8], ev_c);
    atomicAdd(&C->prof[9], ev_nodes);
  }
  if (tid == 0) {
    atomicAdd(&C->prof[0], t_work);
    atomicAdd(&C->prof[5], s_acc[0]);
    atomicAdd(&C->prof[6], (unsigned long long)(k - k_begin));
    for (int l = 0; l < 4; ++l) { atomicAdd(&C->prof[10 + l], s_acc[1 + l]); atomicAdd(&C->prof[14 + l], s_acc[5 + l]); }
  }
}

// ------------------------------------------------------------------ NoTracking
// Every point every step (src/Run.cpp:428-444): T_last = T, T = Calc_T(set); a point that
// was liquid and no longer is gets a record.
template <int PREC>
__global__ void __launch_bounds__(256) k_notrack(DevProblem P, TrackState S, NodeWindow W, int k) {
  __shared__ float4 sA[256], sB[256], sC[256];
  __shared__ int s_liq;
  if (__ldcg(&S.C->done)) return;
  const int slot = k - W.base + 1;
  const NodeBufView nb = slot_view(W, slot);
  const int nn = W.count[slot];
  const double t = W.t[slot];
  if (threadIdx.x == 0) s_liq = 0;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = p < P.pnum;
  double x = 0, y = 0, z = 0;
  if (live) point_xyz(P, p, x, y, z);
  double sum = 0.0;
  if (PREC == 0) {
    for (int n = 0; n < nn; ++n) {
      const double dx = x - __ldg(nb.x + n), dy = y - __ldg(nb.y + n), dz = z - __ldg(nb.z + n);
      sum += __ldg(nb.dtau + n) * __ldg(nb.amp + n) *
             exp(-3.0 * (dx * dx * __ldg(nb.ipx + n) + dy * dy * __ldg(nb.ipy + n) + dz * dz * __ldg(nb.ipz + n)));
    }
  } else {
    const float xh = __double2float_rn(x), yh = __double2float_rn(y), zh = __double2float_rn(z);
    const float xl = __double2float_rn(x - (double)xh), yl = __double2float_rn(y - (double)yh),
                zl = __double2float_rn(z - (double)zh);
    float s = 0.f, c = 0.f;
    for (int base = 0; base < nn; base += 256) {
      __syncthreads();
      const int idx = base + threadIdx.x;
      if (idx < nn) {
        sA[threadIdx.x] = make_float4(nb.xh[idx], nb.xl[idx], nb.yh[idx], nb.yl[idx]);
        sB[threadIdx.x] = make_float4(nb.zh[idx], nb.zl[idx], nb.kx[idx], nb.ky[idx]);
        sC[threadIdx.x] = make_float4(nb.kz[idx], nb.w[idx], 0.f, 0.f);
      }
      __syncthreads();
      const int m = min(256, nn - base);
      for (int j = 0; j < m; ++j) {
        const float4 a = sA[j], b = sB[j], cc = sC[j];
        const float dx = (xh - a.x) + (xl - a.y), dy = (yh - a.z) + (yl - a.w), dz = (zh - b.x) + (zl - b.y);
        const float v = ex2_approx(fmaf(dz * dz, cc.x, fmaf(dy * dy, b.w, dx * dx * b.z))) * cc.y;
        const float yy = v - c;
        const float tt = s + yy;
        c = (tt - s) - yy;
        s = tt;
      }
    }
    sum = (double)s - (double)c;
    // within the guard band of T_L the liquid decision is taken on the FP64 sum (as in tracking)
    if (live && fabs(P.T0 + sum - P.TL) < (double)kGuardRel * (P.TL - P.T0)) {
      double s64 = 0.0;
      for (int n = 0; n < nn; ++n) {
        const double dx = x - __ldg(nb.x + n), dy = y - __ldg(nb.y + n), dz = z - __ldg(nb.z + n);
        s64 += __ldg(nb.dtau + n) * __ldg(nb.amp + n) *
               exp(-3.0 * (dx * dx * __ldg(nb.ipx + n) + dy * dy * __ldg(nb.ipy + n) + dz * dz * __ldg(nb.ipz + n)));
      }
      sum = s64;
    }
  }
  __syncthreads();
  if (live) {
    const double Tprev = S.T[p];
    const double T = P.T0 + sum;
    S.T_last[p] = Tprev;
    S.T[p] = T;
    if (T >= P.TL) {
      S.outflag[p] = 1;
      S.last_liq[p] = k;
      atomicAdd(&s_liq, 1);
    } else if (Tprev >= P.TL) {
      push_record(S, (int)p, k, t, T, Tprev);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_liq) atomicAdd(&S.C->liq_n[0], s_liq);
    if (blockIdx.x == 0) atomicAdd(S.pairs, (unsigned long long)nn * (unsigned long long)P.pnum);
  }
}

__global__ void k_notrack_finish(DevProblem P, TrackState S, NodeWindow W, int k) {
  TrackCounters* C = S.C;
  if (C->done) return;
  const double t = W.t[k - W.base + 1];
  C->step = k + 1;
  if (t > P.end_time && C->liq_n[0] == 0) C->done = 1;
  C->liq_n[0] = 0;
}

// ------------------------------------------------------------------ bulk solidification
// The sums of Grid::Solidify at one point; the FP32 form also returns the magnitudes its
// gradient and Laplacian terms add up to (sum |seg| (|dpx| + |dpy| + |dpz|) and
// sum |seg| (dp^2 - dd)), which bound how far FP32 term errors can move the results.
struct PointSums { double T, gx, gy, gz, lap, dtt, g_mag, lap_mag; };

// Every node of the list at time t, one thread walking the path serially (the same walk as
// gen_list_warp, nodes in the reference's order, image copies applied node by node).
template <bool GRAD>
__device__ __forceinline__ void point_sums(const DevProblem& P, double x, double y, double z, double t, bool is_sol, PointSums& o,
                           unsigned long long& pairs, int& err) {
  o.T = o.gx = o.gy = o.gz = o.lap = o.dtt = o.g_mag = o.lap_mag = 0.0;
  auto add = [&](const NodeVal& v) {
    for (int im = 0; im < P.n_images; ++im) {
      double nx = v.x, ny = v.y, nz = v.z;
      if (im) {
        nx = image_coord(P.img[im][0], P.bcx0, P.bcx1, v.x);
        ny = image_coord(P.img[im][1], P.bcy0, P.bcy1, v.y);
        nz = image_coord(P.img[im][2], P.bcz0, P.bcz1, v.z);
      }
      const double dx = x - nx, dy = y - ny, dz = z - nz;
      const double phi = v.amp * exp(-3.0 * ((dx * dx * v.ipx) + (dy * dy * v.ipy) + (dz * dz * v.ipz)));
      const double seg = v.dtau * phi;
      o.T += seg;
      if (GRAD) {
        const double ddx = -6.0 * v.ipx, ddy = -6.0 * v.ipy, ddz = -6.0 * v.ipz;
        const double dpx = ddx * dx, dpy = ddy * dy, dpz = ddz * dz;
        o.gx += seg * dpx; o.gy += seg * dpy; o.gz += seg * dpz;
        o.lap += seg * (dpx * dpx + dpy * dpy + dpz * dpz + ddx + ddy + ddz);
        o.dtt += (v.dtau == 0) ? phi : 0.0;
      }
      ++pairs;
    }
  };
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    Walk W;
    walk_begin(B, path, t, is_sol, W);
    NodeVal v;
    if (instant_node(P, B, path, W, v)) add(v);
    int steps = 0;
    while (W.more) {
      if (++steps > kMaxWalkSteps) { err |= ERR_WALK_LIMIT; break; }
      walk_interval(B, path, W);
      const int base = W.order - 2;
      for (int kk = base + W.order - 1; kk >= base; --kk)
        if (gauss_node(P, B, path, W, kk, v)) add(v);
      walk_advance(W);
    }
  }
}

// The FP64 sums of point_sums by one warp: every lane walks the path (the walk's
// arithmetic is the same in all lanes) and the lanes share each interval's Gauss nodes,
// lane l taking node l; the lanes' partial sums are reduced at the end, so every lane
// returns the sums.  Warp-collective.
template <bool GRAD>
__device__ __forceinline__ void point_sums_warp(const DevProblem& P, double x, double y, double z, double t,
                                                bool is_sol, PointSums& o, unsigned long long& pairs, int& err) {
  const int lane = threadIdx.x & 31;
  double s[6] = {0, 0, 0, 0, 0, 0};
  auto add = [&](const NodeVal& v) {
    for (int im = 0; im < P.n_images; ++im) {
      double nx = v.x, ny = v.y, nz = v.z;
      if (im) {
        nx = image_coord(P.img[im][0], P.bcx0, P.bcx1, v.x);
        ny = image_coord(P.img[im][1], P.bcy0, P.bcy1, v.y);
        nz = image_coord(P.img[im][2], P.bcz0, P.bcz1, v.z);
      }
      const double dx = x - nx, dy = y - ny, dz = z - nz;
      const double phi = v.amp * exp(-3.0 * ((dx * dx * v.ipx) + (dy * dy * v.ipy) + (dz * dz * v.ipz)));
      const double seg = v.dtau * phi;
      s[0] += seg;
      if (GRAD) {
        const double ddx = -6.0 * v.ipx, ddy = -6.0 * v.ipy, ddz = -6.0 * v.ipz;
        const double dpx = ddx * dx, dpy = ddy * dy, dpz = ddz * dz;
        s[1] += seg * dpx; s[2] += seg * dpy; s[3] += seg * dpz;
        s[4] += seg * (dpx * dpx + dpy * dpy + dpz * dpz + ddx + ddy + ddz);
        s[5] += (v.dtau == 0) ? phi : 0.0;
      }
      ++pairs;
    }
  };
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    Walk W;
    walk_begin(B, path, t, is_sol, W);
    NodeVal v;
    if (lane == 0 && instant_node(P, B, path, W, v)) add(v);
    int steps = 0;
    while (W.more) {
      if (++steps > kMaxWalkSteps) { err |= ERR_WALK_LIMIT; break; }
      walk_interval(B, path, W);
      if (lane < W.order && gauss_node(P, B, path, W, W.order - 2 + lane, v)) add(v);
      walk_advance(W);
    }
  }
#pragma unroll
  for (int j = 0; j < 6; ++j)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s[j] += __shfl_xor_sync(0xffffffffu, s[j], off);
  o.T = s[0]; o.gx = s[1]; o.gy = s[2]; o.gz = s[3]; o.lap = s[4]; o.dtt = s[5];
  o.g_mag = o.lap_mag = 0.0;
}

// The same sums in the FP32 form.  The walk stays FP64, and so do each node's time before
// t (t - t') and its offset from the point; the inverse widths, amplitude, exponential and the
// six sums (Kahan-compensated) are FP32.  FP64 arithmetic issues at about 1/64 of the FP32
// rate on this GPU, so per node only the time and the three offsets are formed in FP64, each
// one fused multiply-add from constants of its interval: t - t' = (t - m) - (h/2) x_k and
// offset = (x - p0 - r0 D) - (h/2 D / duration) x_k for a line segment (m the interval's
// midpoint, x_k the Gauss abscissa, p0 and D the segment's start and extent, r0 the
// midpoint's fraction along it).  The power cut-off box is tested once per interval when
// both ends of the segment lie inside it (the nodes lie between them), else per node exactly
// as the reference computes the position; image copies mirror the node in FP64.
template <bool GRAD>
__device__ __forceinline__ void point_sums_f32(const DevProblem& P, double x, double y, double z, double t, bool is_sol,
                               PointSums& o, unsigned long long& pairs, int& err) {
  float s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0, c0 = 0, c1 = 0, c2 = 0, c3 = 0, c4 = 0, c5 = 0;
  float m_g = 0.f, m_lap = 0.f;             // magnitudes (positive terms: plain sums suffice)
  auto kahan = [](float& sj, float& cj, float v) {
    const float yy = v - cj, tt = sj + yy;
    cj = (tt - sj) - yy;
    sj = tt;
  };
  const float a12f = (float)P.a12;
  // a node at FP64 offset (ox, oy, oz) from the point, tau before t, with power q beta (qb)
  // and weight dtau (0: the instantaneous node)
  auto add = [&](double ox, double oy, double oz, float tau, float qb, float dtau, float ax2, float ay2, float az2) {
    const float ct = a12f * tau;
    const float fx = ax2 + ct, fy = ay2 + ct, fz = az2 + ct;
    const float ipx = __frcp_rn(fx), ipy = __frcp_rn(fy), ipz = __frcp_rn(fz);
    const float amp = qb * __frsqrt_rn(fx * fy * fz);
    for (int im = 0; im < P.n_images; ++im) {
      float dx = (float)ox, dy = (float)oy, dz = (float)oz;
      if (im) {                                  // the mirrored node, from its FP64 position
        dx = (float)(x - image_coord(P.img[im][0], P.bcx0, P.bcx1, x - ox));
        dy = (float)(y - image_coord(P.img[im][1], P.bcy0, P.bcy1, y - oy));
        dz = (float)(z - image_coord(P.img[im][2], P.bcz0, P.bcz1, z - oz));
      }
      const float e = (float)kNeg3Log2e * ((dx * dx * ipx + dy * dy * ipy) + dz * dz * ipz);
      const float phi = amp * ex2_approx(e);
      const float seg = dtau * phi;
      kahan(s0, c0, seg);
      if (GRAD) {
        const float ddx = -6.f * ipx, ddy = -6.f * ipy, ddz = -6.f * ipz;
        const float dpx = ddx * dx, dpy = ddy * dy, dpz = ddz * dz;
        kahan(s1, c1, seg * dpx); kahan(s2, c2, seg * dpy); kahan(s3, c3, seg * dpz);
        const float dp2 = (dpx * dpx + dpy * dpy) + dpz * dpz, dd = (ddx + ddy) + ddz;
        kahan(s4, c4, seg * (dp2 + dd));
        if (dtau == 0.f) kahan(s5, c5, phi);
        m_g += seg * ((fabsf(dpx) + fabsf(dpy)) + fabsf(dpz));
        m_lap += seg * (dp2 - dd);
      }
      ++pairs;
    }
  };
  auto inside = [&](double px, double py) {    // strictly inside the cut-off box, with a margin
    const double mx = 1e-9 * (fabs(P.rx0) + fabs(P.rx1)), my = 1e-9 * (fabs(P.ry0) + fabs(P.ry1));
    return px < P.rx1 - mx && px > P.rx0 + mx && py < P.ry1 - my && py > P.ry0 + my;
  };
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    const float ax2 = (float)B.ax2, ay2 = (float)B.ay2, az2 = (float)B.az2;
    Walk W;
    walk_begin(B, path, t, is_sol, W);
    {
      const BeamLoc L = beam_loc(P, path, W.t, W.s);
      const double qb = L.q * B.beta;
      if (W.t <= B.tlast && qb > 0.0) add(x - L.x, y - L.y, z - L.z, 0.f, (float)qb, 0.f, ax2, ay2, az2);
    }
    int steps = 0;
    while (W.more) {
      if (++steps > kMaxWalkSteps) { err |= ERR_WALK_LIMIT; break; }
      walk_interval(B, path, W);
      const DevSeg cur = path[W.s], prv = path[W.s - 1];
      const double h = W.t2 - W.t1, hh = 0.5 * h;
      if (!(h > 0.0)) { walk_advance(W); continue; }      // zero weights: no node is kept
      const double A = W.t - 0.5 * (W.t2 + W.t1);          // t minus the interval's midpoint
      const int base = W.order - 2;
      const bool line = !cur.mode;
      // the nodes' offsets: constant for a spot, linear in the abscissa along a line
      double Bx = x - cur.x, By = y - cur.y, Bz = z - cur.z, Cx = 0.0, Cy = 0.0, Cz = 0.0, inv = 0.0;
      if (line) {
        inv = 1.0 / (cur.tend - prv.tend);
        const double r0 = (0.5 * (W.t2 + W.t1) - prv.tend) * inv, r1 = hh * inv;
        const double DX = cur.x - prv.x, DY = cur.y - prv.y, DZ = cur.z - prv.z;
        Bx = (x - prv.x) - r0 * DX; By = (y - prv.y) - r0 * DY; Bz = (z - prv.z) - r0 * DZ;
        Cx = r1 * DX; Cy = r1 * DY; Cz = r1 * DZ;
      }
      const bool all_in = line ? (inside(cur.x, cur.y) && inside(prv.x, prv.y)) : inside(cur.x, cur.y);
      const float qb_in = (float)(cur.q * B.beta), hhf = (float)hh;
      if (all_in && !(cur.q * B.beta > 0.0)) { walk_advance(W); continue; }
      for (int kk = base + W.order - 1; kk >= base; --kk) {
        const double loc = P.gl_loc[kk];
        float qb = qb_in;
        if (!all_in) {                                     // the reference's per-node test
          const double tp = 0.5 * (h * loc + (W.t2 + W.t1));
          double lx = cur.x, ly = cur.y;
          if (line) {
            const double r = (tp - prv.tend) * inv;
            lx = prv.x + r * (cur.x - prv.x); ly = prv.y + r * (cur.y - prv.y);
          }
          const bool out = (lx > P.rx1) || (lx < P.rx0) || (ly > P.ry1) || (ly < P.ry0);
          if (out || !(cur.q * B.beta > 0.0)) continue;
        }
        add(fma(-Cx, loc, Bx), fma(-Cy, loc, By), fma(-Cz, loc, Bz), (float)fma(-hh, loc, A), qb,
            hhf * (float)P.gl_w[kk], ax2, ay2, az2);
      }
      walk_advance(W);
    }
  }
  o.T = (double)s0 - (double)c0;
  o.gx = (double)s1 - (double)c1;
  o.gy = (double)s2 - (double)c2;
  o.gz = (double)s3 - (double)c3;
  o.lap = (double)s4 - (double)c4;
  o.dtt = (double)s5 - (double)c5;
  o.g_mag = m_g;
  o.lap_mag = m_lap;
}

// C int abs() applied to a double (the reference's int abs on doubles, src/Grid.cpp:381,535),
// with the x86-64 conversion result INT_MIN for values outside int.
__device__ __forceinline__ double int_abs(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return -2147483648.0;
  const int i = (int)x;
  if (i == INT_MIN) return -2147483648.0;
  return (double)(i < 0 ? -i : i);
}

__global__ void k_sol_latest(TrackState S, const SolRec* rec, int nrec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nrec) atomicMax(&S.sol_step[rec[i].p], rec[i].step);
}

// The reference's secant step for the solidification time from (t - dt, T1) and (t, T2)
// (src/Grid.cpp:340-404; with its int abs() the search stops after the first iteration).
template <int PREC>
__device__ __forceinline__ double secant_tsol(const DevProblem& P, double x, double y, double z, double T2, double T1,
                                              double t, unsigned long long& pairs, int& err) {
  double t2 = t, t1 = rn_sub(t, P.dt), tsol = 0.0;
  PointSums ps;
  for (int it = 1;; ++it) {
    const double m = rn_div(rn_sub(T2, T1), rn_sub(t2, t1));
    tsol = rn_add(t1, rn_div(rn_sub(P.TL, T1), m));
    if (PREC == 0) point_sums<false>(P, x, y, z, tsol, false, ps, pairs, err);
    else point_sums_f32<false>(P, x, y, z, tsol, false, ps, pairs, err);
    const double Tt = P.T0 + ps.T;
    const double e = int_abs(rn_sub(1.0, rn_div(Tt, P.TL)));
    if ((e < P.sol_tol) || (it >= P.sol_iter)) break;
    if (Tt > P.TL) { t1 = tsol; T1 = Tt; } else { t2 = tsol; T2 = Tt; }
  }
  return tsol;
}

// The first estimate of the reference's secant (its only one in practice, see below).
__device__ __forceinline__ double secant_first(const DevProblem& P, double T2, double T1, double t) {
  const double t1 = rn_sub(t, P.dt);
  const double m = rn_div(rn_sub(T2, T1), rn_sub(t, t1));
  return rn_add(t1, rn_div(rn_sub(P.TL, T1), m));
}

// The reference's secant stops after its first estimate when its test value, int abs of
// 1 - T(t_sol) / T_L with T from the plain node schedule (src/Grid.cpp:366-401), is below
// Sol_Tol - which for a positive Sol_Tol happens exactly when 0 < T(t_sol) < 2 T_L - or when
// Sol_Iter is 1.  The gradient sums at the same t_sol give T on the refined schedule, which
// differs from the plain one by the quadrature error (~1e-3 relative); when that T lies
// more than kStopMargin T_L inside (0, 2 T_L), the test's outcome is certain and the plain
// schedule's sum is not formed.  Otherwise the secant runs as the reference's does.
constexpr double kStopMargin = 0.05;
__device__ __forceinline__ bool stop_test_decided(const DevProblem& P, double T_refined) {
  if (P.sol_iter <= 1) return true;
  return P.sol_tol > 0.0 && T_refined > kStopMargin * P.TL && T_refined < (2.0 - kStopMargin) * P.TL;
}

// G, the unit gradient, dT/dt (the reference's int abs), V and eqFrac of point p from the
// gradient sums at tsol (src/Grid.cpp:522-548), stored in the output fields.
__device__ __forceinline__ double cool_rate(const DevProblem& P, const PointSums& ps) {
  return int_abs(rn_add(rn_mul(P.a, ps.lap), ps.dtt));
}

__device__ __forceinline__ void store_fields(const DevProblem& P, const TrackState& S, int p, double tsol,
                                             const PointSums& ps) {
  const double G = sqrt(ps.gx * ps.gx + ps.gy * ps.gy + ps.gz * ps.gz);
  const double dTdt = cool_rate(P, ps);
  const double V = dTdt / G;
  const double kPi = 3.14159265358979323846;
  const double eq = 1.0 - exp((-4 * kPi * P.cetN0 / 3) * pow(G * (P.cetn + 1) / (pow(P.ceta * V, 1 / P.cetn)), -3.0));
  if (S.tSol) S.tSol[p] = tsol;
  if (S.G) S.G[p] = G;
  if (S.Gx) S.Gx[p] = ps.gx / G;
  if (S.Gy) S.Gy[p] = ps.gy / G;
  if (S.Gz) S.Gz[p] = ps.gz / G;
  if (S.dTdt) S.dTdt[p] = dTdt;
  if (S.V) S.V[p] = V;
  if (S.eqFrac) S.eqFrac[p] = eq;
}

// FP32 runs hand a record's solidification to the FP64 redo pass (which takes the secant's
// two temperatures and every sum in FP64) when FP32 arithmetic could miss the fields'
// 1e-4 relative accuracy:
//  - kCondMax: the gradient or cooling-rate terms add up to more than kCondMax times the
//    result (they cancel); FP32 terms are good to about 1e-6 relative, so the results of the
//    rest are good to about 3e-5;
//  - kSecantMinK, kSensMax: the solidification time moves by dt * e / |T2 - T1| for an error
//    e in either secant temperature (kTempErr (T_L - T_0) for FP32 sums near the liquidus:
//    2e-4 K on the benchmark decks), and the cooling rate, a sum that cancels by its
//    condition number c, moves with it roughly in proportion to c.  Records with |T2 - T1|
//    below kSecantMinK or c * dt * e / |T2 - T1| above kSensMax (seconds) are redone.  The
//    bound was set on the 500 x 500 x 100 Surface deck: shifting every point's
//    solidification time by the largest FP32 error leaves the rest within 1.8e-5 relative,
//    and 1.4 % of the records are redone.
constexpr double kCondMax = 32.0;
constexpr double kSecantMinK = 1.0;
constexpr double kTempErr = 1.5e-7;
constexpr double kSensMax = 4e-9;

// Solidification time by the reference's secant step, then gradient, Laplacian and source
// sums at that time with the refined schedule, and the derived fields (src/Grid.cpp:316-548).
// FIX: the second FP32 pass, over the records queued for FP64 temperatures only (k_fix_T has
// summed T and T_last in FP64): the secant then starts exactly as the FP64 form's does, and
// the record goes on to the full FP64 redo only if its sums cancel or the stop test needs the
// secant's FP32 iterations.
template <int PREC, bool FIX>
__global__ void __launch_bounds__(128, 4) k_solidify(DevProblem P, TrackState S, const SolRec* rec, int nrec) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (FIX ? min(__ldcg(S.fix_n), S.rec_cap) : nrec)) return;
  const int i = FIX ? S.fix[e].i : e;
  const SolRec r = rec[i];
  // a later record of this point sets its fields; RDF keeps every record's time and rate
  const bool latest = S.sol_step[r.p] == r.step;
  if (!latest && S.rdf_sol == nullptr) return;
  double x, y, z;
  point_xyz(P, r.p, x, y, z);
  unsigned long long pairs = 0;
  int err = 0;
  const double T2 = FIX ? S.fix_T[e].x : t_decode(S, P, r.T), T1 = FIX ? S.fix_T[e].y : t_decode(S, P, r.Tl);
  double tsol = secant_first(P, T2, T1, r.t);
  PointSums ps;
  if (PREC == 0) point_sums<true>(P, x, y, z, tsol, true, ps, pairs, err);
  else point_sums_f32<true>(P, x, y, z, tsol, true, ps, pairs, err);
  const bool decided = stop_test_decided(P, P.T0 + ps.T);
  if (!decided) {                                    // the secant as the reference runs it
    const double ts = secant_tsol<PREC>(P, x, y, z, T2, T1, r.t, pairs, err);
    if (ts != tsol) {
      tsol = ts;
      if (PREC == 0) point_sums<true>(P, x, y, z, tsol, true, ps, pairs, err);
      else point_sums_f32<true>(P, x, y, z, tsol, true, ps, pairs, err);
    }
  }
  if (PREC != 0) {
    const double G = sqrt(ps.gx * ps.gx + ps.gy * ps.gy + ps.gz * ps.gz);
    const double rate = fabs(rn_add(rn_mul(P.a, ps.lap), ps.dtt));
    const double mag = P.a * ps.lap_mag + ps.dtt, dT = fabs(T2 - T1);
    int why = 0;
    if (!(ps.g_mag <= kCondMax * G) || !(mag <= kCondMax * rate)) why |= 1;
    if (FIX) {
      if (!decided) why |= 2;                        // iterated on FP32 temperatures
    } else if (!(dT >= kSecantMinK) || !(mag * P.dt * kTempErr * (P.TL - P.T0) <= kSensMax * rate * dT)) {
      why |= 2;
    }
    if (!FIX && why == 2) {                          // FP64 temperatures are enough: k_fix_T, then FIX
      const int j = atomicAdd(S.fix_n, 1);
      if (j < S.rec_cap) S.fix[j] = RedoRec{i, why};
    } else if (why) {                                // at most one entry per record: no overflow
      const int j = atomicAdd(S.redo_n, 1);
      if (j < S.rec_cap) S.redo[j] = RedoRec{i, why};
    }
  }
  if (latest) store_fields(P, S, r.p, tsol, ps);
  if (S.rdf_sol) S.rdf_sol[S.rdf_base + i] = RdfSol{r.p, r.step, tsol, cool_rate(P, ps)};
  atomicAdd(S.pairs, pairs);
  atomicAdd(S.pairs + 1, pairs);
  if (err) atomicOr(S.err, err);
}

// FP64 sums of a point over the first nn nodes of a list, by the whole block (each thread a
// strided share of the nodes, then a block reduction); every thread returns the sums.
// `red` holds a block's partial sums (kGenThreads / 32 warps x 6).
template <bool GRAD>
__device__ void block_sums(const NodeBufView& nb, int nn, double x, double y, double z, PointSums& o,
                           double (*red)[6], unsigned long long& pairs) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int n = threadIdx.x; n < nn; n += blockDim.x) {
    const double ipx = nb.ipx[n], ipy = nb.ipy[n], ipz = nb.ipz[n], dtau = nb.dtau[n];
    const double dx = x - nb.x[n], dy = y - nb.y[n], dz = z - nb.z[n];
    const double phi = nb.amp[n] * exp(-3.0 * ((dx * dx * ipx) + (dy * dy * ipy) + (dz * dz * ipz)));
    const double seg = dtau * phi;
    s[0] += seg;
    if (GRAD) {
      const double ddx = -6.0 * ipx, ddy = -6.0 * ipy, ddz = -6.0 * ipz;
      const double dpx = ddx * dx, dpy = ddy * dy, dpz = ddz * dz;
      s[1] += seg * dpx; s[2] += seg * dpy; s[3] += seg * dpz;
      s[4] += seg * (dpx * dpx + dpy * dpy + dpz * dpz + ddx + ddy + ddz);
      s[5] += (dtau == 0) ? phi : 0.0;
    }
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s[j] += __shfl_xor_sync(0xffffffffu, s[j], off);
  }
  __syncthreads();                                  // the previous use of red is over
  if (lane == 0)
    for (int j = 0; j < 6; ++j) red[warp][j] = s[j];
  __syncthreads();
  double t[6] = {0, 0, 0, 0, 0, 0};
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
    for (int j = 0; j < 6; ++j) t[j] += red[w][j];
  o.T = t[0]; o.gx = t[1]; o.gy = t[2]; o.gz = t[3]; o.lap = t[4]; o.dtt = t[5];
  o.g_mag = o.lap_mag = 0.0;
  pairs += threadIdx.x == 0 ? (unsigned long long)nn : 0ull;
}

// point_sums_warp kept out of line (the rare path of block_sums_at).
template <bool GRAD>
__device__ __noinline__ void point_sums_warp_call(const DevProblem* P, double x, double y, double z, double t,
                                                  bool is_sol, PointSums* o, unsigned long long* pairs, int* err) {
  point_sums_warp<GRAD>(*P, x, y, z, t, is_sol, *o, *pairs, *err);
}

// The block's scratch list at time t (one out-of-line copy of the generator for both sums).
__device__ __noinline__ void gen_scratch_list(const DevProblem& P, const TrackState& S, double t, bool is_sol,
                                              GenShared& sh, GenComp* cs) {
  NodeBufView nb = S.redo_nb;
  const size_t off = (size_t)blockIdx.x * S.redo_cap;
  nb.x += off; nb.y += off; nb.z += off; nb.ipx += off; nb.ipy += off; nb.ipz += off; nb.dtau += off; nb.amp += off;
  nb.kx += off; nb.ky += off; nb.kz += off; nb.w += off; nb.xh += off; nb.xl += off; nb.yh += off; nb.yl += off;
  nb.zh += off; nb.zl += off;
  nb.cap = S.redo_cap;
  int* cnt = S.redo_aux + 2 * blockIdx.x;
  if (threadIdx.x == 0) cnt[1] = 0;
  __syncthreads();
  gen_list_block(P, t, is_sol, nb, cnt, cnt + 1, sh, cs);
  __syncthreads();
}

// Sums at time t from a list generated by the block into its scratch buffer; a list longer
// than the buffer is summed by warp 0 walking the path itself (point_sums_warp) instead, or,
// for a compressing deck (whose walk only the list generator restates), reported as
// ERR_NODE_CAPACITY.
template <bool GRAD>
__device__ void block_sums_at(const DevProblem& P, const TrackState& S, double t, bool is_sol, double x, double y,
                              double z, PointSums& o, GenShared& sh, GenComp* cs, double (*red)[6], PointSums& bc,
                              unsigned long long& pairs, int& err) {
  NodeBufView nb = S.redo_nb;
  const size_t off = (size_t)blockIdx.x * S.redo_cap;
  nb.x += off; nb.y += off; nb.z += off; nb.ipx += off; nb.ipy += off; nb.ipz += off; nb.dtau += off; nb.amp += off;
  nb.kx += off; nb.ky += off; nb.kz += off; nb.w += off; nb.xh += off; nb.xl += off; nb.yh += off; nb.yl += off;
  nb.zh += off; nb.zl += off;
  nb.cap = S.redo_cap;
  const int* cnt = S.redo_aux + 2 * blockIdx.x;
  gen_scratch_list(P, S, t, is_sol, sh, cs);
  const int n = __ldcg(cnt), e = __ldcg(cnt + 1);
  err |= e & ERR_WALK_LIMIT;
  if (!(e & ERR_NODE_CAPACITY) && n <= nb.cap) {
    block_sums<GRAD>(nb, n, x, y, z, o, red, pairs);
    return;
  }
  if (P.compress) {
    err |= ERR_NODE_CAPACITY;
    o.T = o.gx = o.gy = o.gz = o.lap = o.dtt = o.g_mag = o.lap_mag = 0.0;
    return;
  }
  if (threadIdx.x < 32) {
    PointSums w;
    int e2 = 0;
    unsigned long long pr = 0;
    point_sums_warp_call<GRAD>(&P, x, y, z, t, is_sol, &w, &pr, &e2);
    if (threadIdx.x == 0) { bc = w; pairs += pr; err |= e2; }
  }
  __syncthreads();
  o = bc;
  __syncthreads();
}

// FP64 temperatures of the records the FP32 pass queued for them (S.fix), one thread block
// per record: T and T_last summed in FP64 over the node window's lists of the record's step
// and the step before it - the sums the FP64 redo starts from - for k_solidify's FIX pass.
// A queue that one round of redo blocks takes whole goes to the FP64 redo instead (its
// latency is one record's; the second FP32 pass would add its own on the same stream).
__global__ void __launch_bounds__(kGenThreads, 2) k_fix_T(DevProblem P, TrackState S, NodeWindow W, const SolRec* rec) {
  __shared__ double red[kGenThreads / 32][6];
  __shared__ int s_base;
  const int n = min(__ldcg(S.fix_n), S.rec_cap);
  if (n <= (int)gridDim.x) {
    if (blockIdx.x == 0 && n > 0) {
      if (threadIdx.x == 0) s_base = atomicAdd(S.redo_n, n);
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (s_base + i < S.rec_cap) S.redo[s_base + i] = S.fix[i];
      __syncthreads();
      if (threadIdx.x == 0) *S.fix_n = 0;
    }
    return;
  }
  unsigned long long pairs = 0;
  for (int e = blockIdx.x; e < n; e += gridDim.x) {
    const SolRec r = rec[S.fix[e].i];
    double x, y, z;
    point_xyz(P, r.p, x, y, z);
    const int slot = r.step - W.base + 1;
    PointSums ps;
    block_sums<false>(slot_view(W, slot), min(W.count[slot], W.slot_cap), x, y, z, ps, red, pairs);
    const double T2 = P.T0 + ps.T;
    block_sums<false>(slot_view(W, slot - 1), min(W.count[slot - 1], W.slot_cap), x, y, z, ps, red, pairs);
    if (threadIdx.x == 0) {
      S.fix_T[e] = make_double2(T2, P.T0 + ps.T);
      atomicAdd(&S.C->fix_total, 1ull);
    }
  }
  if (threadIdx.x == 0 && pairs) { atomicAdd(S.pairs, pairs); atomicAdd(S.pairs + 1, pairs); }
}

// The FP64 redo of the records an FP32 pass queued, one thread block per record: T and
// T_last again in FP64 from the node window's lists of the record's step and the step
// before it (the lists the tracking loop summed in FP32), the reference's secant, and the
// gradient sums at the solidification time from a list the block generates, all in FP64;
// then the fields, overwriting the FP32 pass's values of the record.  The window is intact:
// a window is rebuilt on the same stream only after its records' solidification.
// all > 0: every one of the first `all` records instead of the queue (the solidification of
// compressing decks, whose walk only the list generator restates; a later record of a
// point wins, as in k_solidify).  A compressing deck's kernel takes a GenComp as dynamic
// shared memory.
__global__ void __launch_bounds__(kGenThreads, 2) k_solidify_redo(DevProblem P, TrackState S, NodeWindow W,
                                                                  const SolRec* rec, int all) {
  __shared__ GenShared sh;
  __shared__ double red[kGenThreads / 32][6];
  __shared__ PointSums bc;
  extern __shared__ __align__(16) unsigned char gen_dyn[];
  GenComp* cs = P.compress ? (GenComp*)gen_dyn : nullptr;
  const int n = all > 0 ? all : min(__ldcg(S.redo_n), S.rec_cap);
  unsigned long long pairs = 0;
  int err = 0;
  for (int e = blockIdx.x; e < n; e += gridDim.x) {
    const int ri = all > 0 ? e : S.redo[e].i;
    const SolRec r = rec[ri];
    const bool latest = S.sol_step[r.p] == r.step;
    if (all > 0 && !latest && S.rdf_sol == nullptr) continue;   // block-uniform: a later record wins
    double x, y, z;
    point_xyz(P, r.p, x, y, z);
    const int slot = r.step - W.base + 1;
    PointSums ps;
    block_sums<false>(slot_view(W, slot), min(W.count[slot], W.slot_cap), x, y, z, ps, red, pairs);
    double T2 = P.T0 + ps.T;
    block_sums<false>(slot_view(W, slot - 1), min(W.count[slot - 1], W.slot_cap), x, y, z, ps, red, pairs);
    double T1 = P.T0 + ps.T;
    // the reference's secant (see secant_tsol and stop_test_decided), every sum by the block
    double tsol = secant_first(P, T2, T1, r.t);
    block_sums_at<true>(P, S, tsol, true, x, y, z, ps, sh, cs, red, bc, pairs, err);
    if (!stop_test_decided(P, P.T0 + ps.T)) {
      double t2 = r.t, t1 = rn_sub(r.t, P.dt);
      for (int it = 1;; ++it) {
        const double m = rn_div(rn_sub(T2, T1), rn_sub(t2, t1));
        tsol = rn_add(t1, rn_div(rn_sub(P.TL, T1), m));
        block_sums_at<false>(P, S, tsol, false, x, y, z, ps, sh, cs, red, bc, pairs, err);
        const double Tt = P.T0 + ps.T;
        const double e2 = int_abs(rn_sub(1.0, rn_div(Tt, P.TL)));
        if ((e2 < P.sol_tol) || (it >= P.sol_iter)) break;
        if (Tt > P.TL) { t1 = tsol; T1 = Tt; } else { t2 = tsol; T2 = Tt; }
      }
      block_sums_at<true>(P, S, tsol, true, x, y, z, ps, sh, cs, red, bc, pairs, err);
    }
    if (threadIdx.x == 0) {
      if (latest) store_fields(P, S, r.p, tsol, ps);
      if (S.rdf_sol) S.rdf_sol[S.rdf_base + ri] = RdfSol{r.p, r.step, tsol, cool_rate(P, ps)};
      if (all == 0) atomicAdd(&S.C->redo_total, 1ull);
    }
  }
  if (threadIdx.x == 0) {
    if (pairs) { atomicAdd(S.pairs, pairs); atomicAdd(S.pairs + 1, pairs); }
    if (err) atomicOr(S.err, err);
  }
}

// field ids for k_final_field
enum { F_T, F_TSOL, F_G, F_V, F_GX, F_GY, F_GZ, F_DTDT, F_EQ, F_NUMMELT, F_DEPTH, F_FLAG };

__global__ void k_final_field(DevProblem P, TrackState S, int f, double* out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.pnum) return;
  const bool liquid_last = S.last_liq[p] > S.sol_step[p];
  double v = 0.0;
  switch (f) {
    case F_T: v = t_decode(S, P, S.T[p]); break;
    case F_TSOL: v = S.tSol ? S.tSol[p] : 0.0; break;
    case F_G: v = liquid_last ? DBL_MIN : (S.G ? S.G[p] : 0.0); break;
    case F_V: v = liquid_last ? DBL_MIN : (S.V ? S.V[p] : 0.0); break;
    case F_GX: v = S.Gx ? S.Gx[p] : 0.0; break;
    case F_GY: v = S.Gy ? S.Gy[p] : 0.0; break;
    case F_GZ: v = S.Gz ? S.Gz[p] : 0.0; break;
    case F_DTDT: v = S.dTdt ? S.dTdt[p] : 0.0; break;
    case F_EQ: v = liquid_last ? -1.0 : (S.eqFrac ? S.eqFrac[p] : 0.0); break;
    case F_NUMMELT: v = (double)S.num_melt[p]; break;
    case F_DEPTH: v = S.depth ? rn_mul(S.depth[p], P.hz) : 0.0; break;
    case F_FLAG: v = S.outflag[p] ? 1.0 : 0.0; break;
  }
  out[p] = v;
}

}  // namespace

void th_launch_nodes_window(const DevProblem& P, const NodeWindow& w, int first_slot, int nslots, bool is_sol,
                            int* d_err, cudaStream_t s) {
  if (nslots <= 0) return;
  k_nodes_window<<<nslots, kGenThreads, P.compress ? sizeof(GenComp) : 0, s>>>(P, w, first_slot, nslots, is_sol ? 1 : 0,
                                                                              d_err);
}

// The layout SlotRef reads: every field one array of nb.cap entries, the fields nb.cap apart
// in the order of SlotRef's field enums.
static bool window_layout_ok(const NodeBufView& nb) {
  const double* d[8] = {nb.x, nb.y, nb.z, nb.ipx, nb.ipy, nb.ipz, nb.dtau, nb.amp};
  const float* f[10] = {nb.kx, nb.ky, nb.kz, nb.w, nb.xh, nb.xl, nb.yh, nb.yl, nb.zh, nb.zl};
  for (int i = 0; i < 8; ++i) if (d[i] != nb.x + (size_t)i * nb.cap) return false;
  for (int i = 0; i < 10; ++i) if (f[i] != nb.kx + (size_t)i * nb.cap) return false;
  return true;
}

template <int PREC, int TM>
static cudaError_t launch_track_t(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k_begin, int k_end,
                                  int hw, cudaStream_t s) {
  if (!window_layout_ok(w.nb)) return cudaErrorInvalidValue;
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // stage whole lists up to the slot capacity, within 200 KB of shared memory for the three buffers
  int cap = std::min(w.slot_cap, (200 * 1024) / (3 * staged_bytes_per_node<PREC>()));
  // THESIS_GB300_STAGE_CAP (tests): stage at most this many nodes of a list, so that the
  // passes read the rest from the node window as they do for lists longer than the stage
  if (const char* env = std::getenv("THESIS_GB300_STAGE_CAP")) {
    const int v = std::atoi(env);
    if (v > 0) cap = std::min(cap, v);
  }
  // test knobs of the failure paths: a shorter bound on every wait, and items that are
  // counted into each step but never dealt (the step cannot end; its waits run out)
  long long spin_limit = kSpinLimit;
  int hold = 0;
  if (const char* env = std::getenv("THESIS_GB300_SPIN_LIMIT")) {
    const long long v = std::atoll(env);
    if (v > 0) spin_limit = std::min(v, kSpinLimit);
  }
  if (const char* env = std::getenv("THESIS_GB300_HOLD_ITEMS")) hold = std::max(0, std::atoi(env));
  cap = std::max(kListPad, cap & ~(kListPad - 1));
  const size_t smem = (size_t)3 * cap * staged_bytes_per_node<PREC>() +
                      (axis_in_smem<PREC>(P) ? (size_t)(P.nx + P.ny + P.nz) * sizeof(float2) : 0);
  cudaError_t e = cudaFuncSetAttribute(k_track<PREC, TM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // Shared memory for this block and one k_nodes_window block beside it (the next window's
  // lists are built on the other stream while this one is tracked; without the room that
  // launch waits for the tracking launch to end), the rest of the SM's 256 KB to the L1
  // cache.  A carveout picks the smallest configuration at or above the request.
  cudaFuncAttributes ta{}, na{};
  if ((e = cudaFuncGetAttributes(&ta, k_track<PREC, TM>)) != cudaSuccess) return e;
  if ((e = cudaFuncGetAttributes(&na, k_nodes_window)) != cudaSuccess) return e;
  const size_t need = smem + ta.sharedSizeBytes + na.sharedSizeBytes + (P.compress ? sizeof(GenComp) : 0) +
                      2 * 1024;                                                   // + 1 KB reserved per block
  const int carve = std::min(100, (int)((need * 100 + 228 * 1024 - 1) / (228 * 1024)));
  e = cudaFuncSetAttribute(k_track<PREC, TM>, cudaFuncAttributePreferredSharedMemoryCarveout, carve);
  if (e != cudaSuccess) return e;
  constexpr bool SURF = TM != TM_VOLUME;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_track<PREC, TM>, track_threads<SURF>(), smem);
  const int blocks = sms * (occ < 1 ? occ : 1);
  if (blocks <= 0 || (unsigned)blocks > StepWord<SURF>::kArrMask) return cudaErrorInvalidConfiguration;
  DevProblem Pc = P;
  TrackState Sc = S;
  NodeWindow Wc = w;
  void* args[] = {&Pc, &Sc, &Wc, &k_begin, &k_end, &hw, &cap, &spin_limit, &hold};
  return cudaLaunchCooperativeKernel((const void*)k_track<PREC, TM>, dim3(blocks), dim3(track_threads<SURF>()), args, smem,
                                     s);
}

cudaError_t th_launch_track(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k_begin, int k_end,
                            int precision, int rec_high_water, cudaStream_t s) {
  const int tm = P.tracking == TH_TRACK_STORK                           ? TM_STORK
                 : P.tracking == TH_TRACK_SURFACE && S.rdf_open != nullptr ? TM_SURFACE_RDF
                 : P.tracking == TH_TRACK_SURFACE                         ? TM_SURFACE
                                                                          : TM_VOLUME;
  if (precision == 0) {
    if (tm == TM_STORK) return launch_track_t<0, TM_STORK>(P, S, w, k_begin, k_end, rec_high_water, s);
    if (tm == TM_SURFACE_RDF) return launch_track_t<0, TM_SURFACE_RDF>(P, S, w, k_begin, k_end, rec_high_water, s);
    if (tm == TM_SURFACE) return launch_track_t<0, TM_SURFACE>(P, S, w, k_begin, k_end, rec_high_water, s);
    return launch_track_t<0, TM_VOLUME>(P, S, w, k_begin, k_end, rec_high_water, s);
  }
  if (tm == TM_STORK) return launch_track_t<1, TM_STORK>(P, S, w, k_begin, k_end, rec_high_water, s);
  if (tm == TM_SURFACE_RDF) return launch_track_t<1, TM_SURFACE_RDF>(P, S, w, k_begin, k_end, rec_high_water, s);
  if (tm == TM_SURFACE) return launch_track_t<1, TM_SURFACE>(P, S, w, k_begin, k_end, rec_high_water, s);
  return launch_track_t<1, TM_VOLUME>(P, S, w, k_begin, k_end, rec_high_water, s);
}

void th_launch_notrack_step(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k, int precision,
                            cudaStream_t s) {
  const unsigned blocks = (unsigned)((P.pnum + 255) / 256);
  if (precision == 0) k_notrack<0><<<blocks, 256, 0, s>>>(P, S, w, k);
  else k_notrack<1><<<blocks, 256, 0, s>>>(P, S, w, k);
  k_notrack_finish<<<1, 1, 0, s>>>(P, S, w, k);
}

void th_launch_solidify(const DevProblem& P, const TrackState& S, const NodeWindow& w, const SolRec* rec, int nrec,
                        int precision, bool do_sol, cudaStream_t s) {
  if (nrec <= 0) return;
  k_sol_latest<<<(nrec + 255) / 256, 256, 0, s>>>(S, rec, nrec);
  if (!do_sol) return;
  if (P.compress) {               // every record by the list-based FP64 kernel
    k_solidify_redo<<<S.redo_blocks, kGenThreads, sizeof(GenComp), s>>>(P, S, w, rec, nrec);
    return;
  }
  if (precision == 0) {
    k_solidify<0, false><<<(nrec + 127) / 128, 128, 0, s>>>(P, S, rec, nrec);
    return;
  }
  k_solidify<1, false><<<(nrec + 127) / 128, 128, 0, s>>>(P, S, rec, nrec);
  // records whose secant is too sensitive to FP32 temperatures get FP64 ones (a block each)
  // and a second FP32 pass; those whose sums cancel get the full FP64 redo (a block each): a
  // persistent pass over each queue, then the queues are emptied
  k_fix_T<<<S.redo_blocks, kGenThreads, 0, s>>>(P, S, w, rec);
  k_solidify<1, true><<<(nrec + 127) / 128, 128, 0, s>>>(P, S, rec, nrec);
  k_solidify_redo<<<S.redo_blocks, kGenThreads, 0, s>>>(P, S, w, rec, 0);
  cudaMemsetAsync(S.redo_n, 0, sizeof(int), s);
  cudaMemsetAsync(S.fix_n, 0, sizeof(int), s);
}

void th_launch_final_field(const DevProblem& P, const TrackState& S, int field, double* out, cudaStream_t s) {
  k_final_field<<<(unsigned)((P.pnum + 255) / 256), 256, 0, s>>>(P, S, field, out);
}
