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
__global__ void __launch_bounds__(kGenThreads) k_nodes_window(DevProblem P, NodeWindow w, int first, int n, int is_sol,
                                                              int* err) {
  __shared__ GenShared sh;
  const int slot = first + blockIdx.x;
  const NodeBufView nb = slot_view(w, slot);
  gen_list_block(P, w.t[slot], is_sol != 0, nb, &w.count[slot], err, sh);
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

__device__ __forceinline__ void push_record(const TrackState& S, int p, int step, double t, double T, double Tl) {
  const int i = atomicAdd(S.rec_n, 1);
  if (i < S.rec_cap) { SolRec r; r.p = p; r.step = step; r.t = t; r.T = T; r.Tl = Tl; S.rec[i] = r; }
  else atomicOr(S.err, ERR_RECORDS);
  atomicAdd(&S.num_melt[p], 1);
}

// Grid::Calc_T with set = true (src/Grid.cpp:300-311): the liquid markers (G = V = DBL_MIN,
// eqFrac = -1) are applied when fields are read, from last_liq.
__device__ __forceinline__ void set_T(const TrackState& S, const DevProblem& P, int p, double T, int step) {
  S.T[p] = T;
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
        if (++spins > kSpinLimit) {
          if (atomicOr(S.err, ERR_BARRIER) == 0) { S.C->diag[0] = 2; S.C->diag[2] = (int)blockIdx.x; S.C->diag[4] = (int)*S.bar; }
          break;
        }
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

__device__ __forceinline__ int64_t pid(const DevProblem& P, int i, int j, int k) {
  return (int64_t)i * ((int64_t)P.ny * P.nz) + (int64_t)j * P.nz + k;
}

// Claim for this step (the reference's T_calc_flag test-and-set, src/Melt.cpp:213-218):
// a point counts as claimed in step k when its stamp is >= k + 1.
__device__ __forceinline__ bool claim(const TrackState& S, int q, unsigned stamp) {
  if (__ldcg(S.stamp + q) >= stamp) return false;
  return atomicMax(S.stamp + q, stamp) < stamp;
}

// ------------------------------------------------------------------ step work queue
enum { IT_RETEST = 0, IT_SEEDS = 1, IT_VISIT = 2, IT_COLUMN = 3, IT_DEPTH = 4 };

struct StepCtx {
  int k;                   // step
  unsigned stamp;          // k + 1
  double t;
  NodeBufView nb, nbl;
  int nn, nnl;
  int nL, n_init;
  const int* L;
  int* Lo;
  int* lo_n;
  QueueCounters* qc;
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_s32(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Publishes one child item per lane that has one (warp-uniform call).  The children are
// counted as published in the same atomic that hands out their slots, before any of them
// can be taken, so "completed == initial + published" can only hold once the step has no
// work left; each slot's tag is released after its payload.
__device__ __forceinline__ void emit(const TrackState& S, const StepCtx& X, bool has, int type, int p, int aux,
                                     int& nchild) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(0xffffffffu, has);
  if (!m) return;
  unsigned base = 0;
  if (lane == 0) base = (unsigned)(atomicAdd(&X.qc->state, (unsigned long long)__popc(m) << 32) >> 32);
  base = __shfl_sync(0xffffffffu, base, 0);
  if (has) {
    const unsigned j = base + __popc(m & ((1u << lane) - 1u));
    if (j < (unsigned)S.queue_cap) {
      int4* slot = S.queue + j;
      slot->y = type; slot->z = p; slot->w = aux;
      st_release_s32(&slot->x, (int)X.stamp);
    } else {
      atomicOr(S.err, ERR_QUEUE);
    }
  }
  nchild += __popc(m);
}

// Claims the unvisited neighbours of p (3x3 in the same layer for Surface, 3x3x{k-1, k}
// for Volume; src/Melt.cpp:202-257) and queues them for evaluation.
template <bool SURF>
__device__ __forceinline__ void expand(const DevProblem& P, const TrackState& S, const StepCtx& X, int p, int& nchild) {
  const int lane = threadIdx.x & 31;
  const int nyz = P.ny * P.nz;
  const int pi = p / nyz, pj = (p / P.nz) % P.ny, pk = p % P.nz;
  bool got = false;
  int q = 0;
  if (lane < (SURF ? 9 : 18)) {
    const int di = (lane % 9) / 3 - 1, dj = lane % 3 - 1, dk = SURF ? 0 : (lane / 9) - 1;
    const int ni = pi + di, nj = pj + dj, nk = pk + dk;
    if (!(ni < 0 || ni > P.nx - 1 || nj < 0 || nj > P.ny - 1 || nk < 0)) {
      q = (int)pid(P, ni, nj, nk);
      got = claim(S, q, X.stamp);
    }
  }
  emit(S, X, got, IT_VISIT, q, 0, nchild);
}

__device__ __forceinline__ void push_liquid(const TrackState& S, const StepCtx& X, int p) {
  const int i = atomicAdd(X.lo_n, 1);
  if (i < S.list_cap) X.Lo[i] = p; else atomicOr(S.err, ERR_LISTS);
  atomicMax(S.stamp + p, X.stamp + 1u);   // already claimed for the next step's re-test
}

// Perimeter seeds of one anchor point (src/Melt.cpp:36-55, 69-77): when the anchor lies
// outside the grid, surface points along that edge within CheckRadius * ax are tested.
__device__ void perimeter(const DevProblem& P, const TrackState& S, const StepCtx& X, double x, double y, double r2,
                          int& nchild) {
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
    for (int v0 = 0; v0 < hi; v0 += 32) {
      const int v = v0 + lane;
      bool got = false;
      int q = 0;
      if (v < hi) {
        const int i = xfixed ? fixed : v, j = xfixed ? v : fixed;
        const double dx = rn_sub(rn_add(P.xmin, rn_mul((double)i, P.xres)), x);
        const double dy = rn_sub(rn_add(P.ymin, rn_mul((double)j, P.yres)), y);
        if (rn_add(rn_mul(dx, dx), rn_mul(dy, dy)) < r2) {
          q = (int)pid(P, i, j, P.nz - 1);
          got = claim(S, q, X.stamp);
        }
      }
      emit(S, X, got, IT_VISIT, q, 0, nchild);
    }
  }
}

// The 2 x 2 surface cells at and after an anchor inside the grid (src/Melt.cpp:122-146).
__device__ void cell(const DevProblem& P, const TrackState& S, const StepCtx& X, double x, double y, int& nchild) {
  const int lane = threadIdx.x & 31;
  const int xg = (int)floor(rn_div(rn_sub(x, P.xmin), P.xres));
  const int yg = (int)floor(rn_div(rn_sub(y, P.ymin), P.yres));
  if (xg < 0 || xg > P.nx - 1 || yg < 0 || yg > P.ny - 1) return;
  bool got = false;
  int q = 0;
  if (lane < 4) {
    const int i = xg + (lane >> 1), j = yg + (lane & 1);
    if (!(i < 0 || i > P.nx - 1 || j < 0 || j > P.ny - 1)) {
      q = (int)pid(P, i, j, P.nz - 1);
      got = claim(S, q, X.stamp);
    }
  }
  emit(S, X, got, IT_VISIT, q, 0, nchild);
}

// Melt::beam_trace for (t - dt, t] (src/Melt.cpp:20-183), claims queued as visits.
__device__ void beam_trace(const DevProblem& P, const TrackState& S, const StepCtx& X, int& nchild) {
  const double t_end = X.t, t_start = rn_sub(X.t, P.dt);
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam& B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    const double rc2 = rn_mul(P.rcheck, P.rcheck);
    const double tsub = rn_div(rn_mul(rn_sub(rc2, 1.0), B.ax2), rn_mul(12.0, P.a));
    const double ts = (rn_sub(t_end, tsub) < 0.0) ? 0.0 : rn_sub(t_end, tsub);
    const double r2 = rn_mul(rn_mul(rc2, B.ax), B.ax);
    const int s0 = first_ge(path, B.nseg, ts), s1 = first_ge(path, B.nseg, t_end);
    for (int s = max(s0 - 1, 0); s <= s1; ++s) perimeter(P, S, X, path[s].x, path[s].y, r2, nchild);
    if (path[s1].mode == 0 && t_end < B.tlast) {
      const BeamLoc L = beam_loc(P, path, t_end, s1);
      perimeter(P, S, X, L.x, L.y, r2, nchild);
    }
  }
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam& B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    const int s0 = first_ge(path, B.nseg, t_start), s1 = first_ge(path, B.nseg, t_end);
    for (int s = max(s0 - 1, 0); s <= s1; ++s) cell(P, S, X, path[s].x, path[s].y, nchild);
    if (path[s1].mode == 0 && t_end < B.tlast) {
      const BeamLoc L = beam_loc(P, path, t_end, s1);
      cell(P, S, X, L.x, L.y, nchild);
    }
  }
}

// Depth walk under a liquid surface point and the running depth maximum
// (src/Melt.cpp:271-357): walk down while liquid, else walk up solidifying.
template <int PREC>
__device__ void depth_walk(const DevProblem& P, const TrackState& S, const StepCtx& X, int p,
                           unsigned long long& pairs) {
  const int lane = threadIdx.x & 31;
  const int col = p / P.nz;
  const int D = ldcg_i(S.depths + col);
  int d = D;
  bool none_deeper = true;
  while (true) {
    ++d;
    if (d == P.nz) break;
    const int q = col * P.nz + (P.nz - 1 - d);
    const double T = warp_T<PREC>(P, X.nb, X.nn, q);
    pairs += X.nn;
    if (lane == 0) set_T(S, P, q, T, X.k);
    if (!(T >= P.TL)) break;
    none_deeper = false;
  }
  while (true) {
    --d;
    if (d == 0 || !none_deeper) break;
    const int q = col * P.nz + (P.nz - 1 - d);
    const double Told = ldcg_d(S.T + q);
    const double T = warp_T<PREC>(P, X.nb, X.nn, q);
    pairs += X.nn;
    if (lane == 0) set_T(S, P, q, T, X.k);
    if (!(T >= P.TL)) {
      double Tl = Told;                                   // T of the previous step
      if (d != D) { Tl = warp_T<PREC>(P, X.nbl, X.nnl, q); pairs += X.nnl; }
      if (lane == 0) push_record(S, q, X.k, X.t, T, Tl);
    } else {
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
        const double Tl = ldcg_d(S.T + col * P.nz + (P.nz - 1 - d));
        const double Ts = ldcg_d(S.T + col * P.nz + (P.nz - 1 - (d + 1)));
        dep = rn_add((double)d, rn_div(rn_sub(P.TL, Tl), rn_sub(Ts, Tl)));
      }
      if (dep > S.depth_max[col]) {
        S.depth_max[col] = dep;
        for (int dd = d; dd >= 0; --dd) S.depth[col * P.nz + (P.nz - 1 - dd)] = dep;
      }
    }
  }
}

// One work item; returns the number of child items it published (already counted).
template <int PREC, bool SURF>
__device__ int run_item(const DevProblem& P, const TrackState& S, const StepCtx& X, int type, int p, int aux,
                        unsigned long long& pairs) {
  const int lane = threadIdx.x & 31;
  int nchild = 0;
  if (type == IT_SEEDS) {
    beam_trace(P, S, X, nchild);
    return nchild;
  }
  if (type == IT_DEPTH) {
    depth_walk<PREC>(P, S, X, p, pairs);
    return 0;
  }
  const double Told = ldcg_d(S.T + p);
  const double T = warp_T<PREC>(P, X.nb, X.nn, p);
  pairs += X.nn;
  if (lane == 0) set_T(S, P, p, T, X.k);
  const bool liquid = T >= P.TL;
  if (type == IT_COLUMN) {                 // a layer under a surface point that solidified
    double Tl = Told;
    if (aux) { Tl = warp_T<PREC>(P, X.nbl, X.nnl, p); pairs += X.nnl; }
    if (lane == 0) push_record(S, p, X.k, X.t, T, Tl);
    return 0;
  }
  if (type == IT_RETEST && !liquid) {      // cooled below T_L since the last step
    if (lane == 0) push_record(S, p, X.k, X.t, T, Told);
    if (SURF) {
      const int col = p / P.nz;
      const int D = ldcg_i(S.depths + col);
      for (int d0 = 1; d0 <= D; d0 += 32) {
        const int d = d0 + lane;
        emit(S, X, d <= D, IT_COLUMN, col * P.nz + (P.nz - 1 - d), d != D, nchild);
      }
      if (lane == 0) S.depths[col] = 0;
    }
  }
  if (liquid && lane == 0) push_liquid(S, X, p);
  // Surface expands every re-tested point, Volume only the liquid ones (src/Run.cpp:655, 531)
  if (liquid || (SURF && type == IT_RETEST)) expand<SURF>(P, S, X, p, nchild);
  // the depth walk under a liquid surface point needs nothing else from this step
  if (SURF && liquid) depth_walk<PREC>(P, S, X, p, pairs);
  return nchild;
}

// ------------------------------------------------------------------ the tracking loop
constexpr int kTrackThreads = 128;   // four warps per block, one block per SM
// One launch runs steps [k_begin, k_end) of a Volume or Surface loop (src/Run.cpp:469-709).
// Each step is a single phase: the previous step's liquid points are re-tested, the beam
// trace seeds the new ones, and every claimed point, column and depth walk becomes a work
// item that any warp may take; a packed (published << 32 | completed) counter tells the
// warps when the step has no work left, and one grid barrier ends the step.
template <int PREC, bool SURF>
__global__ void __launch_bounds__(kTrackThreads) k_track(DevProblem P, TrackState S, NodeWindow W, int k_begin,
                                                        int k_end, int high_water) {
  const int lane = threadIdx.x & 31;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  TrackCounters* C = S.C;
  unsigned long long pairs = 0;
  for (int k = k_begin; k < k_end; ++k) {
    StepCtx X;
    const int slot = k - W.base + 1;
    X.k = k;
    X.stamp = (unsigned)k + 1u;
    X.nb = slot_view(W, slot);
    X.nbl = slot_view(W, slot - 1);
    X.nn = W.count[slot];
    X.nnl = (k == 0) ? 0 : W.count[slot - 1];
    X.t = W.t[slot];
    const int b0 = k % 3, b1 = (k + 1) % 3, b2 = (k + 2) % 3;
    X.nL = ldcg_i(&C->liq_n[b0]);
    X.L = S.liq[b0];
    X.Lo = S.liq[b1];
    X.lo_n = &C->liq_n[b1];
    X.qc = &C->q[b0];
    const bool seeds = k > 0 && X.t < P.end_time + P.dt;
    X.n_init = X.nL + (seeds ? 1 : 0);
    if (tid == 0) {                       // buffers of the step after next
      C->liq_n[b2] = 0;
      C->q[b1].head = 0; C->q[b1].state = 0ull;
    }
    // the work loop
    long long idle = 0;
    while (true) {
      unsigned ticket = 0;
      if (lane == 0) ticket = atomicAdd(&X.qc->head, 1u);
      ticket = __shfl_sync(0xffffffffu, ticket, 0);
      int type, p = 0, aux = 0;
      if (ticket < (unsigned)X.nL) {
        type = IT_RETEST;
        p = __ldcg(X.L + ticket);
      } else if (ticket < (unsigned)X.n_init) {
        type = IT_SEEDS;
      } else {
        const unsigned j = ticket - (unsigned)X.n_init;
        bool ready = false, finished = false;
        unsigned backoff = 8;
        while (true) {
          if (lane == 0) {
            const int tag = (j < (unsigned)S.queue_cap) ? ld_acquire_s32(&S.queue[j].x) : 0;
            ready = tag == (int)X.stamp;
            if (!ready) {
              const unsigned long long st = ld_relaxed_u64(&X.qc->state);
              finished = (unsigned)(st & 0xffffffffu) == (unsigned)X.n_init + (unsigned)(st >> 32);
            }
          }
          ready = __shfl_sync(0xffffffffu, ready, 0);
          finished = __shfl_sync(0xffffffffu, finished, 0);
          if (ready || finished) break;
          backoff = backoff < 256 ? backoff * 2 : 256;
          if (++idle > kSpinLimit) {
            if (lane == 0) {
              if (atomicOr(S.err, ERR_BARRIER) == 0) {        // first waiter to give up records its view
                const unsigned long long st = ld_relaxed_u64(&X.qc->state);
                int* g = S.C->diag;
                g[0] = 1; g[1] = k; g[2] = (int)ticket; g[3] = X.n_init;
                g[4] = (int)*(volatile unsigned*)&X.qc->head; g[5] = (int)(st >> 32);
                g[6] = (int)(st >> 32); g[7] = (int)(st & 0xffffffffu);
              }
            }
            finished = true;
            break;
          }
          __nanosleep(backoff);
        }
        if (!ready) break;
        const int4 it = __ldcg(S.queue + j);
        type = it.y; p = it.z; aux = it.w;
      }
      run_item<PREC, SURF>(P, S, X, type, p, aux, pairs);
      __threadfence();
      if (lane == 0) atomicAdd(&X.qc->state, 1ull);             // completed
    }
    if (!grid_sync(S)) return;
    // finish test (src/Util.cpp:239-243) and the record queue's high-water mark
    const int nLo = ldcg_i(X.lo_n);
    if (tid == 0) {
      C->step = k + 1;
      const unsigned items = (unsigned)(__ldcg(&X.qc->state) >> 32) + (unsigned)X.n_init;
      if ((int)items > C->max_items) C->max_items = (int)items;
    }
    if (X.t > P.end_time && nLo == 0) { if (tid == 0) C->done = 1; break; }
    if (ldcg_i(S.rec_n) > high_water) { if (tid == 0) C->stop = 1; break; }
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

__global__ void k_sol_latest(TrackState S, const SolRec* rec, int nrec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nrec) atomicMax(&S.sol_step[rec[i].p], rec[i].step);
}

// Solidification time by the reference's secant step, then gradient, Laplacian and source
// sums at that time with the refined schedule, and the derived fields (src/Grid.cpp:316-548).
__global__ void __launch_bounds__(128) k_solidify(DevProblem P, TrackState S, const SolRec* rec, int nrec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const SolRec r = rec[i];
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
  k_nodes_window<<<nslots, kGenThreads, 0, s>>>(P, w, first_slot, nslots, is_sol ? 1 : 0, d_err);
}

template <int PREC, bool SURF>
static cudaError_t launch_track_t(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k_begin, int k_end,
                                  int hw, cudaStream_t s) {
  int dev = 0, sms = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_track<PREC, SURF>, kTrackThreads, 0);
  const int blocks = sms * (occ < 1 ? occ : 1);
  if (blocks <= 0) return cudaErrorInvalidConfiguration;
  DevProblem Pc = P;
  TrackState Sc = S;
  NodeWindow Wc = w;
  void* args[] = {&Pc, &Sc, &Wc, &k_begin, &k_end, &hw};
  return cudaLaunchCooperativeKernel((const void*)k_track<PREC, SURF>, dim3(blocks), dim3(kTrackThreads), args, 0, s);
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

void th_launch_solidify(const DevProblem& P, const TrackState& S, const SolRec* rec, int nrec, int precision,
                        bool do_sol, cudaStream_t s) {
  (void)precision;
  if (nrec <= 0) return;
  k_sol_latest<<<(nrec + 255) / 256, 256, 0, s>>>(S, rec, nrec);
  if (do_sol) k_solidify<<<(nrec + 127) / 128, 128, 0, s>>>(P, S, rec, nrec);
}

void th_launch_final_field(const DevProblem& P, const TrackState& S, int field, double* out, cudaStream_t s) {
  k_final_field<<<(unsigned)((P.pnum + 255) / 256), 256, 0, s>>>(P, S, field, out);
}
