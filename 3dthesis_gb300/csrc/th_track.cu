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
#include <cfloat>
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "th_device.cuh"
#include "th_track.h"

using namespace thdev;

namespace {

__device__ __forceinline__ NodeBufView slot_view(const NodeWindow& w, int slot) {
  NodeBufView v = w.nb;
  const size_t off = (size_t)slot * w.slot_cap;
  v.x += off; v.y += off; v.z += off; v.ipx += off; v.ipy += off; v.ipz += off; v.dtau += off; v.amp += off;
  v.kx += off; v.ky += off; v.kz += off; v.w += off; v.xh += off; v.xl += off; v.yh += off; v.yl += off;
  v.zh += off; v.zl += off;
  v.cap = w.slot_cap;
  return v;
}

// ------------------------------------------------------------------ node windows
__global__ void __launch_bounds__(256) k_nodes_window(DevProblem P, NodeWindow w, int first, int n, int is_sol,
                                                      int* err) {
  const int slot = first + (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (slot >= first + n) return;
  const NodeBufView nb = slot_view(w, slot);
  gen_list_warp(P, w.t[slot], is_sol != 0, nb, &w.count[slot], err);
}

// ------------------------------------------------------------------ warp evaluation
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// T at point p from one node list, the 32 lanes of a warp splitting the nodes; every lane
// returns the same value.
template <int PREC>
__device__ __forceinline__ double warp_T(const DevProblem& P, const NodeBufView& nb, int nn, int64_t p) {
  const int lane = threadIdx.x & 31;
  double x, y, z;
  point_xyz(P, p, x, y, z);
  double part;
  if (PREC == 0) {
    double s = 0.0;
    for (int n = lane; n < nn; n += 32) {
      const double dx = x - __ldg(nb.x + n), dy = y - __ldg(nb.y + n), dz = z - __ldg(nb.z + n);
      s += __ldg(nb.dtau + n) * __ldg(nb.amp + n) *
           exp(-3.0 * (dx * dx * __ldg(nb.ipx + n) + dy * dy * __ldg(nb.ipy + n) + dz * dz * __ldg(nb.ipz + n)));
    }
    part = s;
  } else {
    const float xh = __double2float_rn(x), yh = __double2float_rn(y), zh = __double2float_rn(z);
    const float xl = __double2float_rn(x - (double)xh), yl = __double2float_rn(y - (double)yh),
                zl = __double2float_rn(z - (double)zh);
    float s = 0.f, c = 0.f;
    for (int n = lane; n < nn; n += 32) {
      const float dx = (xh - __ldg(nb.xh + n)) + (xl - __ldg(nb.xl + n));
      const float dy = (yh - __ldg(nb.yh + n)) + (yl - __ldg(nb.yl + n));
      const float dz = (zh - __ldg(nb.zh + n)) + (zl - __ldg(nb.zl + n));
      const float e = fmaf(dz * dz, __ldg(nb.kz + n), fmaf(dy * dy, __ldg(nb.ky + n), dx * dx * __ldg(nb.kx + n)));
      const float v = ex2_approx(e) * __ldg(nb.w + n);
      const float yy = v - c;
      const float tt = s + yy;
      c = (tt - s) - yy;
      s = tt;
    }
    part = (double)s - (double)c;
  }
  return P.T0 + warp_sum_d(part);
}

__device__ __forceinline__ int ldcg_i(const int* p) { return __ldcg(p); }
__device__ __forceinline__ double ldcg_d(const double* p) { return __ldcg(p); }

__device__ __forceinline__ void push(int* list, int* cnt, int cap, int v, int* err) {
  const int i = atomicAdd(cnt, 1);
  if (i < cap) list[i] = v; else atomicOr(err, ERR_LISTS);
}

__device__ __forceinline__ void push_record(const TrackState& S, int p, int step, double t, double T, double Tl) {
  const int i = atomicAdd(&S.C->rec_n, 1);
  if (i < S.rec_cap) { SolRec r; r.p = p; r.step = step; r.t = t; r.T = T; r.Tl = Tl; S.rec[i] = r; }
  else atomicOr(S.err, ERR_RECORDS);
  atomicAdd(&S.num_melt[p], 1);
}

// Grid::Calc_T with set = true (src/Grid.cpp:300-311): the liquid markers (G = V = DBL_MIN,
// eqFrac = -1) are applied when fields are read, from last_liq.
__device__ __forceinline__ void set_T(const TrackState& S, const DevProblem& P, int p, double T, int step) {
  S.T[p] = T;
  S.flag[p] = 1u;
  if (T >= P.TL) { S.outflag[p] = 1; S.last_liq[p] = step; }
}

// Grid-wide barrier for the cooperative launch.  The wait is bounded: after kSpinLimit
// polls it latches ERR_BARRIER and every block leaves the kernel at its next check.
constexpr long long kSpinLimit = 1ll << 25;

__device__ __forceinline__ bool grid_sync(const TrackState& S) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = S.bar + 1;
    const unsigned g = *gen;
    __threadfence();
    if (atomicAdd(S.bar, 1u) == gridDim.x - 1) {
      atomicExch(S.bar, 0u);
      __threadfence();
      atomicAdd(S.bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*gen == g) {
        if (++spins > kSpinLimit) { atomicOr(S.err, ERR_BARRIER); break; }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return (*(volatile int*)S.err & ERR_BARRIER) == 0;
}

__device__ __forceinline__ int first_ge(const DevSeg* path, int ns, double t) {
  int lo = 0, hi = ns - 1;                 // first s with t_end >= t, clamped to the last
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (path[mid].tend < t) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void claim_seed(const TrackState& S, int64_t q) {
  if (atomicCAS(&S.flag[q], 0u, 1u) == 0u) push(S.seeds, &S.C->seed_n, S.list_cap, (int)q, S.err);
}

__device__ __forceinline__ int64_t pid(const DevProblem& P, int i, int j, int k) {
  return (int64_t)i * ((int64_t)P.ny * P.nz) + (int64_t)j * P.nz + k;
}

// Perimeter seeds of one anchor point (src/Melt.cpp:36-55, 69-77): when the anchor lies
// outside the grid, surface points along that edge within CheckRadius * ax are tested.
__device__ void perimeter(const DevProblem& P, const TrackState& S, double x, double y, double r2) {
  const int lane = threadIdx.x & 31;
  const int xg = (int)floor(rn_div(rn_sub(x, P.xmin), P.xres));
  const int yg = (int)floor(rn_div(rn_sub(y, P.ymin), P.yres));
  for (int edge = 0; edge < 4; ++edge) {
    int fixed;
    bool xfixed;
    if (edge == 0) { if (!(xg < 0)) continue; fixed = 0; xfixed = true; }
    else if (edge == 1) { if (!(xg > P.nx - 1)) continue; fixed = P.nx - 1; xfixed = true; }
    else if (edge == 2) { if (!(yg < 0)) continue; fixed = 0; xfixed = false; }
    else { if (!(yg > P.ny - 1)) continue; fixed = P.ny - 1; xfixed = false; }
    const int hi = xfixed ? P.ny : P.nx;
    for (int v = lane; v < hi; v += 32) {
      const int i = xfixed ? fixed : v, j = xfixed ? v : fixed;
      const double dx = rn_sub(rn_add(P.xmin, rn_mul((double)i, P.xres)), x);
      const double dy = rn_sub(rn_add(P.ymin, rn_mul((double)j, P.yres)), y);
      if (rn_add(rn_mul(dx, dx), rn_mul(dy, dy)) < r2) claim_seed(S, pid(P, i, j, P.nz - 1));
    }
  }
}

// The 2 x 2 surface cells at and after an anchor inside the grid (src/Melt.cpp:122-146).
__device__ void cell(const DevProblem& P, const TrackState& S, double x, double y) {
  const int lane = threadIdx.x & 31;
  const int xg = (int)floor(rn_div(rn_sub(x, P.xmin), P.xres));
  const int yg = (int)floor(rn_div(rn_sub(y, P.ymin), P.yres));
  if (xg < 0 || xg > P.nx - 1 || yg < 0 || yg > P.ny - 1) return;
  if (lane < 4) {
    const int i = xg + (lane >> 1), j = yg + (lane & 1);
    if (!(i < 0 || i > P.nx - 1 || j < 0 || j > P.ny - 1)) claim_seed(S, pid(P, i, j, P.nz - 1));
  }
}

// Melt::beam_trace for (t_start, t_end], run by one warp (src/Melt.cpp:20-183).
__device__ void beam_trace(const DevProblem& P, const TrackState& S, double t_start, double t_end) {
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam& B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    const double rc2 = rn_mul(P.rcheck, P.rcheck);
    const double tsub = rn_div(rn_mul(rn_sub(rc2, 1.0), B.ax2), rn_mul(12.0, P.a));
    const double ts = (rn_sub(t_end, tsub) < 0.0) ? 0.0 : rn_sub(t_end, tsub);
    const double r2 = rn_mul(rn_mul(rc2, B.ax), B.ax);
    const int s0 = first_ge(path, B.nseg, ts), s1 = first_ge(path, B.nseg, t_end);
    for (int s = max(s0 - 1, 0); s <= s1; ++s) perimeter(P, S, path[s].x, path[s].y, r2);
    if (path[s1].mode == 0 && t_end < B.tlast) {
      const BeamLoc L = beam_loc(P, path, t_end, s1);
      perimeter(P, S, L.x, L.y, r2);
    }
  }
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam& B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    const int s0 = first_ge(path, B.nseg, t_start), s1 = first_ge(path, B.nseg, t_end);
    for (int s = max(s0 - 1, 0); s <= s1; ++s) cell(P, S, path[s].x, path[s].y);
    if (path[s1].mode == 0 && t_end < B.tlast) {
      const BeamLoc L = beam_loc(P, path, t_end, s1);
      cell(P, S, L.x, L.y);
    }
  }
  __syncwarp();
}

// ------------------------------------------------------------------ the tracking loop
template <int PREC, bool SURF>
__global__ void __launch_bounds__(256) k_track(DevProblem P, TrackState S, NodeWindow W, int k_begin, int k_end,
                                               int high_water) {
  const int lane = threadIdx.x & 31;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
  const int warp = tid >> 5, nwarps = nthreads >> 5;
  TrackCounters* C = S.C;
  unsigned long long pairs = 0;
  const int nyz = P.ny * P.nz;
  for (int k = k_begin; k < k_end; ++k) {
    const int slot = k - W.base + 1;
    const NodeBufView nb = slot_view(W, slot), nbl = slot_view(W, slot - 1);
    const int nn = W.count[slot], nnl = (k == 0) ? 0 : W.count[slot - 1];
    const double t = W.t[slot];
    const int cur = k & 1, nxt = cur ^ 1;
    const int nL = ldcg_i(&C->liq_n[cur]), nR = ldcg_i(&C->reset_n[cur]);
    const int* L = S.liq[cur];
    const int* R = S.reset[cur];
    int* Lo = S.liq[nxt];
    int* Ro = S.reset[nxt];
    int* liq_out = &C->liq_n[nxt];
    int* reset_out = &C->reset_n[nxt];

    // A. reset the points evaluated last step; the new reset list starts as last step's
    //    liquid list (src/Run.cpp:603-616)
    for (int i = tid; i < nR; i += nthreads) {
      const int p = __ldcg(R + i);
      S.T_last[p] = ldcg_d(S.T + p);
      S.flag[p] = 0u;
    }
    for (int i = tid; i < nL; i += nthreads) Ro[i] = __ldcg(L + i);
    if (tid == 0) {
      const int prev_rounds = C->rounds;
      for (int r = 0; r <= prev_rounds + 1 && r <= kMaxFrontRounds; ++r) C->front_n[r] = 0;
      *liq_out = 0;
      *reset_out = nL;
      C->col_n = 0;
      C->seed_n = 0;
    }
    if (!grid_sync(S)) return;

    // B. re-test last step's liquid points; queue the ones that cooled below T_L
    for (int i = warp; i < nL; i += nwarps) {
      const int p = __ldcg(L + i);
      const double T = warp_T<PREC>(P, nb, nn, p);
      pairs += nn;
      if (lane == 0) set_T(S, P, p, T, k);
      if (!(T >= P.TL)) {
        if (lane == 0) push_record(S, p, k, t, T, ldcg_d(S.T_last + p));
        if (SURF) {                                  // the column below solidifies too
          const int col = p / P.nz;
          const int D = ldcg_i(S.depths + col);
          for (int d = D - lane; d > 0; d -= 32) {
            const int q = col * P.nz + (P.nz - 1 - d);
            const int w = atomicAdd(&C->col_n, 1);
            if (w < S.list_cap) S.colwork[w] = make_int2(q, d != D); else atomicOr(S.err, ERR_LISTS);
          }
          if (lane == 0) S.depths[col] = 0;
        }
      } else if (lane == 0) {
        push(Lo, liq_out, S.list_cap, p, S.err);
      }
    }
    if (!grid_sync(S)) return;

    // C. column solidification, beam-trace seeds, first frontier
    {
      const int ncol = ldcg_i(&C->col_n);
      for (int i = warp; i < ncol; i += nwarps) {
        const int2 it = __ldcg(S.colwork + i);
        const int q = it.x;
        const double T = warp_T<PREC>(P, nb, nn, q);
        pairs += nn;
        double Tl;
        if (it.y) { Tl = warp_T<PREC>(P, nbl, nnl, q); pairs += nnl; }
        else Tl = ldcg_d(S.T_last + q);
        if (lane == 0) {
          set_T(S, P, q, T, k);
          if (it.y) S.T_last[q] = Tl;
          push_record(S, q, k, t, T, Tl);
          push(Ro, reset_out, S.list_cap, q, S.err);
        }
      }
      if (SURF) {
        for (int i = tid; i < nL; i += nthreads) S.front[0][i] = __ldcg(L + i);
        if (tid == 0) C->front_n[0] = nL;
      } else {
        const int nLo = ldcg_i(liq_out);
        for (int i = tid; i < nLo; i += nthreads) S.front[0][i] = __ldcg(Lo + i);
        if (tid == 0) C->front_n[0] = nLo;
      }
      if (warp == nwarps - 1 && k > 0 && t < P.end_time + P.dt) beam_trace(P, S, rn_sub(t, P.dt), t);
    }
    if (!grid_sync(S)) return;

    // D. evaluate the seeds (src/Run.cpp:662-669)
    {
      const int ns = ldcg_i(&C->seed_n);
      for (int i = warp; i < ns; i += nwarps) {
        const int p = __ldcg(S.seeds + i);
        const double T = warp_T<PREC>(P, nb, nn, p);
        pairs += nn;
        if (lane == 0) {
          set_T(S, P, p, T, k);
          push(Ro, reset_out, S.list_cap, p, S.err);
          if (T >= P.TL) {
            push(S.front[0], &C->front_n[0], S.list_cap, p, S.err);
            push(Lo, liq_out, S.list_cap, p, S.err);
          }
        }
      }
    }
    if (!grid_sync(S)) return;

    // E. frontier rounds: claim unvisited neighbours, evaluate, keep the liquid ones
    //    (src/Melt.cpp:185-269; 3x3 at the same layer for Surface, 3x3x{k-1,k} for Volume)
    int r = 0;
    while (true) {
      const int n_in = ldcg_i(&C->front_n[r]);
      if (n_in == 0) break;
      if (r >= kMaxFrontRounds) { if (tid == 0) atomicOr(S.err, ERR_ROUNDS); break; }
      const int* Fin = S.front[r & 1];
      int* Fout = S.front[(r + 1) & 1];
      int* fout_n = &C->front_n[r + 1];
      for (int i = warp; i < n_in; i += nwarps) {
        const int p = __ldcg(Fin + i);
        const int pi = p / nyz, pj = (p / P.nz) % P.ny, pk = p % P.nz;
        bool claimed = false;
        int q = 0;
        const int nnb = SURF ? 9 : 18;
        if (lane < nnb) {
          const int di = (lane % 9) / 3 - 1, dj = lane % 3 - 1, dk = SURF ? 0 : (lane / 9) - 1;
          const int ni = pi + di, nj = pj + dj, nk = pk + dk;
          if (!(ni < 0 || ni > P.nx - 1 || nj < 0 || nj > P.ny - 1 || nk < 0)) {
            q = (int)pid(P, ni, nj, nk);
            if (__ldcg((const unsigned*)S.flag + q) == 0u) claimed = atomicCAS(&S.flag[q], 0u, 1u) == 0u;
          }
        }
        unsigned m = __ballot_sync(0xffffffffu, claimed);
        while (m) {
          const int src = __ffs(m) - 1;
          m &= m - 1;
          const int qq = __shfl_sync(0xffffffffu, q, src);
          const double T = warp_T<PREC>(P, nb, nn, qq);
          pairs += nn;
          if (lane == 0) {
            set_T(S, P, qq, T, k);
            push(Ro, reset_out, S.list_cap, qq, S.err);
            if (T >= P.TL) {
              push(Fout, fout_n, S.list_cap, qq, S.err);
              push(Lo, liq_out, S.list_cap, qq, S.err);
            }
          }
        }
      }
      if (!grid_sync(S)) return;
      ++r;
    }
    if (tid == 0) { C->rounds = r; if (r > C->max_rounds) C->max_rounds = r; }

    if (SURF && P.nz != 1) {
      // F. depth walk under every liquid surface point (src/Melt.cpp:271-317)
      const int nLo = ldcg_i(liq_out);
      for (int i = warp; i < nLo; i += nwarps) {
        const int p = __ldcg(Lo + i);
        const int col = p / P.nz;
        const int D = ldcg_i(S.depths + col);
        int d = D;
        bool none_deeper = true;
        while (true) {
          ++d;
          if (d == P.nz) break;
          const int q = col * P.nz + (P.nz - 1 - d);
          const double T = warp_T<PREC>(P, nb, nn, q);
          pairs += nn;
          if (lane == 0) { set_T(S, P, q, T, k); push(Ro, reset_out, S.list_cap, q, S.err); }
          if (!(T >= P.TL)) break;
          none_deeper = false;
        }
        while (true) {
          --d;
          if (d == 0 || !none_deeper) break;
          const int q = col * P.nz + (P.nz - 1 - d);
          const double T = warp_T<PREC>(P, nb, nn, q);
          pairs += nn;
          if (lane == 0) { set_T(S, P, q, T, k); push(Ro, reset_out, S.list_cap, q, S.err); }
          if (!(T >= P.TL)) {
            double Tl;
            if (d != D) { Tl = warp_T<PREC>(P, nbl, nnl, q); pairs += nnl; }
            else Tl = ldcg_d(S.T_last + q);
            if (lane == 0) {
              if (d != D) S.T_last[q] = Tl;
              push_record(S, q, k, t, T, Tl);
            }
          } else {
            break;
          }
        }
        if (d == P.nz) --d;
        if (lane == 0) S.depths[col] = d;
      }
      if (!grid_sync(S)) return;
      // G. deepest liquid position per column, kept as a running maximum (src/Melt.cpp:319-357)
      if (S.depth) {
        for (int i = tid; i < nLo; i += nthreads) {
          const int p = __ldcg(Lo + i);
          const int col = p / P.nz;
          const int dl = ldcg_i(S.depths + col);
          double dep;
          if (dl == P.nz - 1) dep = dl;
          else {
            const double Tl = ldcg_d(S.T + col * P.nz + (P.nz - 1 - dl));
            const double Ts = ldcg_d(S.T + col * P.nz + (P.nz - 1 - (dl + 1)));
            dep = rn_add((double)dl, rn_div(rn_sub(P.TL, Tl), rn_sub(Ts, Tl)));
          }
          if (dep > S.depth_max[col]) {
            S.depth_max[col] = dep;
            for (int d = dl; d >= 0; --d) S.depth[col * P.nz + (P.nz - 1 - d)] = dep;
          }
        }
        if (!grid_sync(S)) return;
      }
    }
    // finish test (src/Util.cpp:239-243) and the record queue's high-water mark
    const int nLo = ldcg_i(liq_out);
    if (tid == 0) C->step = k + 1;
    if (t > P.end_time && nLo == 0) { if (tid == 0) C->done = 1; break; }
    if (ldcg_i(&C->rec_n) > high_water) { if (tid == 0) C->stop = 1; break; }
  }
  if (lane == 0 && pairs) atomicAdd(S.pairs, pairs);
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
struct PointSums { double T, gx, gy, gz, lap, dtt; };

// Every node of the list at time t, one thread walking the path serially (the same walk as
// gen_list_warp, nodes in the reference's order, image copies applied node by node).
template <bool GRAD>
__device__ void point_sums(const DevProblem& P, double x, double y, double z, double t, bool is_sol, PointSums& o,
                           unsigned long long& pairs, int& err) {
  o.T = o.gx = o.gy = o.gz = o.lap = o.dtt = 0.0;
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

// C int abs() applied to a double (the reference's int abs on doubles, src/Grid.cpp:381,535),
// with the x86-64 conversion result INT_MIN for values outside int.
__device__ __forceinline__ double int_abs(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return -2147483648.0;
  const int i = (int)x;
  if (i == INT_MIN) return -2147483648.0;
  return (double)(i < 0 ? -i : i);
}

__global__ void k_sol_latest(TrackState S, int nrec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nrec) atomicMax(&S.sol_step[S.rec[i].p], S.rec[i].step);
}

// Solidification time by the reference's secant step, then gradient, Laplacian and source
// sums at that time with the refined schedule, and the derived fields (src/Grid.cpp:316-548).
__global__ void __launch_bounds__(128) k_solidify(DevProblem P, TrackState S, int nrec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const SolRec r = S.rec[i];
  if (S.sol_step[r.p] != r.step) return;            // a later record of this point wins
  double x, y, z;
  point_xyz(P, r.p, x, y, z);
  unsigned long long pairs = 0;
  int err = 0;
  double T2 = r.T, T1 = r.Tl, t2 = r.t, t1 = rn_sub(r.t, P.dt), tsol = 0.0;
  PointSums ps;
  for (int it = 1;; ++it) {
    const double m = rn_div(rn_sub(T2, T1), rn_sub(t2, t1));
    tsol = rn_add(t1, rn_div(rn_sub(P.TL, T1), m));
    point_sums<false>(P, x, y, z, tsol, false, ps, pairs, err);
    const double Tt = P.T0 + ps.T;
    const double e = int_abs(rn_sub(1.0, rn_div(Tt, P.TL)));
    if ((e < P.sol_tol) || (it >= P.sol_iter)) break;
    if (Tt > P.TL) { t1 = tsol; T1 = Tt; } else { t2 = tsol; T2 = Tt; }
  }
  point_sums<true>(P, x, y, z, tsol, true, ps, pairs, err);
  const double G = sqrt(ps.gx * ps.gx + ps.gy * ps.gy + ps.gz * ps.gz);
  const double dTdt = int_abs(rn_add(rn_mul(P.a, ps.lap), ps.dtt));
  const double V = dTdt / G;
  const double kPi = 3.14159265358979323846;
  const double eq = 1.0 - exp((-4 * kPi * P.cetN0 / 3) * pow(G * (P.cetn + 1) / (pow(P.ceta * V, 1 / P.cetn)), -3.0));
  const int p = r.p;
  if (S.tSol) S.tSol[p] = tsol;
  if (S.G) S.G[p] = G;
  if (S.Gx) S.Gx[p] = ps.gx / G;
  if (S.Gy) S.Gy[p] = ps.gy / G;
  if (S.Gz) S.Gz[p] = ps.gz / G;
  if (S.dTdt) S.dTdt[p] = dTdt;
  if (S.V) S.V[p] = V;
  if (S.eqFrac) S.eqFrac[p] = eq;
  atomicAdd(S.pairs, pairs);
  atomicAdd(S.pairs + 1, pairs);
  if (err) atomicOr(S.err, err);
}

// field ids for k_final_field
enum { F_T, F_TSOL, F_G, F_V, F_GX, F_GY, F_GZ, F_DTDT, F_EQ, F_NUMMELT, F_DEPTH, F_FLAG };

__global__ void k_final_field(DevProblem P, TrackState S, int f, double* out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.pnum) return;
  const bool liquid_last = S.last_liq[p] > S.sol_step[p];
  double v = 0.0;
  switch (f) {
    case F_T: v = S.T[p]; break;
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
  const int blocks = (nslots + 7) / 8;
  k_nodes_window<<<blocks, 256, 0, s>>>(P, w, first_slot, nslots, is_sol ? 1 : 0, d_err);
}

template <int PREC, bool SURF>
static cudaError_t launch_track_t(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k_begin, int k_end,
                                  int hw, cudaStream_t s) {
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_track<PREC, SURF>, 256, 0);
  const int blocks = sms * (occ < 2 ? occ : 2);
  if (blocks <= 0) return cudaErrorInvalidConfiguration;
  DevProblem Pc = P;
  TrackState Sc = S;
  NodeWindow Wc = w;
  void* args[] = {&Pc, &Sc, &Wc, &k_begin, &k_end, &hw};
  return cudaLaunchCooperativeKernel((const void*)k_track<PREC, SURF>, dim3(blocks), dim3(256), args, 0, s);
}

cudaError_t th_launch_track(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k_begin, int k_end,
                            int precision, int rec_high_water, cudaStream_t s) {
  const bool surf = P.tracking == TH_TRACK_SURFACE;
  if (precision == 0) return surf ? launch_track_t<0, true>(P, S, w, k_begin, k_end, rec_high_water, s)
                                  : launch_track_t<0, false>(P, S, w, k_begin, k_end, rec_high_water, s);
  return surf ? launch_track_t<1, true>(P, S, w, k_begin, k_end, rec_high_water, s)
              : launch_track_t<1, false>(P, S, w, k_begin, k_end, rec_high_water, s);
}

void th_launch_notrack_step(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k, int precision,
                            cudaStream_t s) {
  const unsigned blocks = (unsigned)((P.pnum + 255) / 256);
  if (precision == 0) k_notrack<0><<<blocks, 256, 0, s>>>(P, S, w, k);
  else k_notrack<1><<<blocks, 256, 0, s>>>(P, S, w, k);
  k_notrack_finish<<<1, 1, 0, s>>>(P, S, w, k);
}

void th_launch_solidify(const DevProblem& P, const TrackState& S, int nrec, int precision, bool do_sol, cudaStream_t s) {
  (void)precision;
  if (nrec <= 0) return;
  k_sol_latest<<<(nrec + 255) / 256, 256, 0, s>>>(S, nrec);
  if (do_sol) k_solidify<<<(nrec + 127) / 128, 128, 0, s>>>(P, S, nrec);
}

void th_launch_final_field(const DevProblem& P, const TrackState& S, int field, double* out, cudaStream_t s) {
  k_final_field<<<(unsigned)((P.pnum + 255) / 256), 256, 0, s>>>(P, S, field, out);
}
