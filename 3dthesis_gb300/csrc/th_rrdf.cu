// Stork's doubly reduced data (RRDF) on the device, built per step from the tracking
// loop's log of liquid columns.
//
// Reference behaviour restated here (3DThesis tree):
//   Run::Stork, the cell pass and the vertex temperatures     src/Run.cpp:958-1071
//   Grid::get_RRDF_idxs / _ts / _Ts (the rows' layout)         src/Grid.h:368-370
//
// A point is liquid at step k when its column's top point is in the step's liquid list
// and the point lies at or above the column's depth (src/Run.cpp:950-955).  The reference
// counts the liquid vertices of every cell (cx*cy*cz cells) at every step that has liquid;
// a cell gets a row when the count changed or is neither 0 nor 8 at this or the previous
// step.  Every such cell has a liquid vertex at one of the two steps, so it lies in a
// cell column (ci, cj) next to a liquid column, and within that column the rows form one
// run of layers: ck from cz - 1 - Dmax (the lowest layer with a liquid vertex) to
// cz - 1 - Dmin (the lowest layer that is not liquid throughout at both steps), Dmax / Dmin
// the largest / smallest depth of the cell column's four vertex columns over the two
// steps (-1 where a column is not liquid).  So a step's rows come from its two liquid
// lists alone: one block per step gathers the cell columns next to the listed columns,
// sorts them (the reference's single-thread row order is ascending cell index), counts
// each column's run, and evaluates every vertex the rows need once per time.
//
// The vertex temperatures are T(vertex, t_k) and T(vertex, t_{k-1}) on the node lists of
// the two steps (the reference computes or reuses exactly these, src/Run.cpp:1024-1040;
// at step 0 the previous values are the initial T_0).
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "th_device.cuh"
#include "th_track.h"

using namespace thdev;

namespace {

constexpr int kRThreads = 256;
constexpr int kSortSmem = 4096;           // candidate lists up to this length are sorted in shared memory
constexpr int kVertsPerThread = 4;

__host__ __device__ inline int pow2_at_least(int v, int lo) {
  int c = lo;
  while (c < v) c <<= 1;
  return c;
}

// Per-block scratch, laid out for lists of up to nmax entries (both lists of a step):
// column hash (keys, depth at k - 1, depth at k), candidate cell columns, the sorted
// unique cell columns with their row runs, and per (cell column, corner) pair the vertex
// column's owner, value offset and layer range.
struct Layout {
  int cap1, scap;
  size_t keys, dp, dc, sort, u, lo, hi, row, pv, po, pl, ph, total;
};

__host__ __device__ inline Layout layout_for(int nmax) {
  Layout L;
  L.cap1 = pow2_at_least(2 * nmax, 32);
  L.scap = pow2_at_least(4 * nmax, 32);
  size_t o = 0;
  L.keys = o; o += L.cap1;
  L.dp = o; o += L.cap1;
  L.dc = o; o += L.cap1;
  L.sort = o; o += L.scap;
  L.u = o; o += L.scap;
  L.lo = o; o += L.scap;
  L.hi = o; o += L.scap;
  L.row = o; o += L.scap;
  L.pv = o; o += 4 * (size_t)L.scap;
  L.po = o; o += 4 * (size_t)L.scap;
  L.pl = o; o += 4 * (size_t)L.scap;
  L.ph = o; o += 4 * (size_t)L.scap;
  L.total = o;
  return L;
}

// Exclusive scan of a[0, n) in place; every thread returns the total.
__device__ int block_scan(int* a, int n, int* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int per = (n + kRThreads - 1) / kRThreads;
  const int b = min(n, (int)threadIdx.x * per), e = min(n, b + per);
  int sum = 0;
  for (int i = b; i < e; ++i) sum += a[i];
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) sh[wid] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int w = 0; w < kRThreads / 32; ++w) { const int v = sh[w]; sh[w] = run; run += v; }
    sh[kRThreads / 32] = run;
  }
  __syncthreads();
  int run = sh[wid] + incl - sum;
  for (int i = b; i < e; ++i) { const int v = a[i]; a[i] = run; run += v; }
  const int total = sh[kRThreads / 32];
  __syncthreads();
  return total;
}

// Ascending bitonic sort of a[0, n), n a power of two.
__device__ void block_sort(int* a, int n) {
  for (int k = 2; k <= n; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n; i += kRThreads) {
        const int x = i ^ j;
        if (x > i) {
          const int ai = a[i], ax = a[x];
          if ((ai > ax) == ((i & k) == 0)) { a[i] = ax; a[x] = ai; }
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ unsigned hash_slot(int key, int cap) {
  return ((unsigned)key * 0x9E3779B1u) & (unsigned)(cap - 1);
}

__device__ int hash_insert(int* keys, int cap, int key) {
  unsigned h = hash_slot(key, cap);
  while (true) {
    const int old = atomicCAS(keys + h, -1, key);
    if (old == -1 || old == key) return (int)h;
    h = (h + 1) & (unsigned)(cap - 1);
  }
}

__device__ int hash_find(const int* keys, int cap, int key) {
  unsigned h = hash_slot(key, cap);
  while (true) {
    const int k = keys[h];
    if (k == key) return (int)h;
    if (k == -1) return -1;
    h = (h + 1) & (unsigned)(cap - 1);
  }
}

// Index of cc in the sorted u[0, n), or -1.
__device__ __forceinline__ int find_sorted(const int* u, int n, int cc) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (u[m] < cc) lo = m + 1; else hi = m;
  }
  return (lo < n && u[lo] == cc) ? lo : -1;
}

struct StepShape {
  int nu;      // cell columns next to a liquid column
  int rows;    // rows of the step
  int nv;      // vertex values per time
};

// Steps 1-7 of a step's build (see the file comment): leaves the sorted cell columns, their
// row runs and row offsets, and the vertex pairs with their owners and value offsets in
// the block's scratch.
__device__ StepShape build_step(const DevProblem& P, const RrdfBatch& B, int j, int* X, const Layout& L, int* s_sort,
                                int* sh) {
  StepShape r{0, 0, 0};
  const int cx = P.nx - 1, cy = P.ny - 1, cz = P.nz - 1;
  const int a0 = B.off[j], a1 = B.off[j + 1], b1 = B.off[j + 2];
  const int na = a1 - a0, n = b1 - a0;
  if (n == 0 || cx < 1 || cy < 1 || cz < 1) return r;
  const int cap1 = pow2_at_least(2 * n, 32), scap = pow2_at_least(4 * n, 32);
  int* keys = X + L.keys; int* dp = X + L.dp; int* dc = X + L.dc;
  int* U = X + L.u; int* lo = X + L.lo; int* hi = X + L.hi; int* row = X + L.row;
  int* pv = X + L.pv; int* po = X + L.po; int* pl = X + L.pl; int* ph = X + L.ph;
  for (int i = threadIdx.x; i < cap1; i += kRThreads) { keys[i] = -1; dp[i] = -1; dc[i] = -1; }
  __syncthreads();
  // 1. depth of every listed column at k - 1 (list j) and at k (list j + 1)
  for (int e = threadIdx.x; e < n; e += kRThreads) {
    const int2 v = B.log[a0 + e];
    const int h = hash_insert(keys, cap1, v.x / P.nz);
    if (e < na) dp[h] = v.y; else dc[h] = v.y;
  }
  // 2. the cell columns next to them, sorted
  int* srt = scap <= kSortSmem ? s_sort : X + L.sort;
  for (int e = threadIdx.x; e < scap / 4; e += kRThreads) {
    int c4[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
    if (e < n) {
      const int col = B.log[a0 + e].x / P.nz;
      const int i = col / P.ny, jj = col % P.ny;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int ci = i - 1 + (q >> 1), cj = jj - 1 + (q & 1);
        if (ci >= 0 && ci < cx && cj >= 0 && cj < cy) c4[q] = ci * cy + cj;
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) srt[4 * e + q] = c4[q];
  }
  __syncthreads();
  block_sort(srt, scap);
  for (int i = threadIdx.x; i < scap; i += kRThreads)
    row[i] = (srt[i] != INT_MAX && (i == 0 || srt[i] != srt[i - 1])) ? 1 : 0;
  __syncthreads();
  const int nu = block_scan(row, scap, sh);
  for (int i = threadIdx.x; i < scap; i += kRThreads)
    if (srt[i] != INT_MAX && (i == 0 || srt[i] != srt[i - 1])) U[row[i]] = srt[i];
  __syncthreads();
  // 3. each cell column's run of rows
  for (int u = threadIdx.x; u < nu; u += kRThreads) {
    const int cc = U[u], ci = cc / cy, cj = cc % cy;
    int dmax = -1, dmin = INT_MAX;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int h = hash_find(keys, cap1, (ci + (q >> 1)) * P.ny + (cj + (q & 1)));
      const int d0 = h < 0 ? -1 : dp[h], d1 = h < 0 ? -1 : dc[h];
      dmax = max(dmax, max(d0, d1));
      dmin = min(dmin, min(d0, d1));
    }
    const int l = max(0, cz - 1 - dmax), t = min(cz - 1, cz - 1 - dmin);
    lo[u] = l; hi[u] = t;
    row[u] = max(0, t - l + 1);
  }
  __syncthreads();
  const int rows = block_scan(row, nu, sh);
  // 4. the vertex columns: each is evaluated once, by the first cell column (in row order)
  // with rows that has it as a corner, over the layers all such cell columns need
  for (int pr = threadIdx.x; pr < 4 * nu; pr += kRThreads) {
    const int u = pr >> 2, c = pr & 3;
    const int cnt = (u + 1 < nu ? row[u + 1] : rows) - row[u];
    int own = -1, vlo = INT_MAX, vhi = -1;
    if (cnt > 0) {
      const int cc = U[u], vi = cc / cy + (c >> 1), vj = cc % cy + (c & 1);
#pragma unroll
      for (int q = 0; q < 4; ++q) {              // (vi-1, vj-1), (vi-1, vj), (vi, vj-1), (vi, vj)
        const int ci = vi - 1 + (q >> 1), cj = vj - 1 + (q & 1);
        if (ci < 0 || ci >= cx || cj < 0 || cj >= cy) continue;
        const int w = find_sorted(U, nu, ci * cy + cj);
        if (w < 0) continue;
        const int cw = (w + 1 < nu ? row[w + 1] : rows) - row[w];
        if (cw <= 0) continue;
        if (own < 0) own = 4 * w + (3 - q);       // v is corner (1 - q>>1, 1 - q&1) of that column
        vlo = min(vlo, lo[w]);
        vhi = max(vhi, hi[w] + 1);
      }
    }
    po[pr] = own;
    pl[pr] = vlo;
    ph[pr] = vhi;
    pv[pr] = (own == pr) ? vhi - vlo + 1 : 0;
  }
  __syncthreads();
  const int nv = block_scan(pv, 4 * nu, sh);
  r.nu = nu; r.rows = rows; r.nv = nv;
  return r;
}

// T_0 + the sum over a step's node list at each of the block's nv vertices (k_notrack's two
// forms: FP64 terms, or FP32 terms with a compensated sum).
template <int PREC>
__device__ void eval_vertices(const DevProblem& P, const NodeWindow& W, int slot, const int* vpt, int nv, double* out,
                              float4* stage) {
  const NodeBufView nb = slot_view(W, slot);
  const int nn = W.count[slot];
  float4* sA = stage;
  float4* sB = stage + kRThreads;
  float4* sC = stage + 2 * kRThreads;
  for (int v0 = 0; v0 < nv; v0 += kRThreads * kVertsPerThread) {
    double x[kVertsPerThread], y[kVertsPerThread], z[kVertsPerThread];
#pragma unroll
    for (int q = 0; q < kVertsPerThread; ++q) {
      const int v = v0 + q * kRThreads + threadIdx.x;
      x[q] = y[q] = z[q] = 0.0;
      if (v < nv) point_xyz(P, vpt[v], x[q], y[q], z[q]);
    }
    double sum[kVertsPerThread];
    if (PREC == 0) {
#pragma unroll
      for (int q = 0; q < kVertsPerThread; ++q) sum[q] = 0.0;
      for (int m = 0; m < nn; ++m) {
        const double nx = __ldg(nb.x + m), ny = __ldg(nb.y + m), nz = __ldg(nb.z + m);
        const double ix = __ldg(nb.ipx + m), iy = __ldg(nb.ipy + m), iz = __ldg(nb.ipz + m);
        const double w = __ldg(nb.dtau + m) * __ldg(nb.amp + m);
#pragma unroll
        for (int q = 0; q < kVertsPerThread; ++q) {
          const double dx = x[q] - nx, dy = y[q] - ny, dz = z[q] - nz;
          sum[q] += w * exp(-3.0 * (dx * dx * ix + dy * dy * iy + dz * dz * iz));
        }
      }
    } else {
      float xh[kVertsPerThread], xl[kVertsPerThread], yh[kVertsPerThread], yl[kVertsPerThread];
      float zh[kVertsPerThread], zl[kVertsPerThread], s[kVertsPerThread], c[kVertsPerThread];
#pragma unroll
      for (int q = 0; q < kVertsPerThread; ++q) {
        xh[q] = __double2float_rn(x[q]); xl[q] = __double2float_rn(x[q] - (double)xh[q]);
        yh[q] = __double2float_rn(y[q]); yl[q] = __double2float_rn(y[q] - (double)yh[q]);
        zh[q] = __double2float_rn(z[q]); zl[q] = __double2float_rn(z[q] - (double)zh[q]);
        s[q] = 0.f; c[q] = 0.f;
      }
      for (int base = 0; base < nn; base += kRThreads) {
        __syncthreads();
        const int idx = base + threadIdx.x;
        if (idx < nn) {
          sA[threadIdx.x] = make_float4(nb.xh[idx], nb.xl[idx], nb.yh[idx], nb.yl[idx]);
          sB[threadIdx.x] = make_float4(nb.zh[idx], nb.zl[idx], nb.kx[idx], nb.ky[idx]);
          sC[threadIdx.x] = make_float4(nb.kz[idx], nb.w[idx], 0.f, 0.f);
        }
        __syncthreads();
        const int m = min(kRThreads, nn - base);
        for (int jn = 0; jn < m; ++jn) {
          const float4 a = sA[jn], b = sB[jn], cc = sC[jn];
#pragma unroll
          for (int q = 0; q < kVertsPerThread; ++q) {
            const float dx = (xh[q] - a.x) + (xl[q] - a.y), dy = (yh[q] - a.z) + (yl[q] - a.w),
                        dz = (zh[q] - b.x) + (zl[q] - b.y);
            const float v = ex2_approx(fmaf(dz * dz, cc.x, fmaf(dy * dy, b.w, dx * dx * b.z))) * cc.y;
            const float yy = v - c[q];
            const float tt = s[q] + yy;
            c[q] = (tt - s[q]) - yy;
            s[q] = tt;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < kVertsPerThread; ++q) sum[q] = (double)s[q] - (double)c[q];
    }
#pragma unroll
    for (int q = 0; q < kVertsPerThread; ++q) {
      const int v = v0 + q * kRThreads + threadIdx.x;
      if (v < nv) out[v] = P.T0 + sum[q];
    }
  }
  __syncthreads();
}

// Count pass: rows and vertex values of each step of the batch.
__global__ void __launch_bounds__(kRThreads) k_rrdf_count(DevProblem P, RrdfBatch B) {
  __shared__ int s_sort[kSortSmem];
  __shared__ int sh[kRThreads / 32 + 1];
  const Layout L = layout_for(B.nmax);
  int* X = B.scratch + (size_t)blockIdx.x * L.total;
  for (int j = blockIdx.x; j < B.nsteps; j += gridDim.x) {
    const StepShape r = build_step(P, B, j, X, L, s_sort, sh);
    if (threadIdx.x == 0) { B.counts[2 * j] = r.rows; B.counts[2 * j + 1] = r.nv; }
    __syncthreads();
  }
}

// Fill pass: the rows of each step at the offsets the host laid out from the counts.
template <int PREC>
__global__ void __launch_bounds__(kRThreads) k_rrdf_fill(DevProblem P, NodeWindow W, RrdfBatch B) {
  __shared__ __align__(16) int s_sort[kSortSmem];       // also the node staging of FP32 evaluations
  __shared__ int sh[kRThreads / 32 + 1];
  const Layout L = layout_for(B.nmax);
  int* X = B.scratch + (size_t)blockIdx.x * L.total;
  double* Tp = B.vals + (size_t)blockIdx.x * 3 * B.vals_cap;
  double* Tc = Tp + B.vals_cap;
  int* vpt = (int*)(Tc + B.vals_cap);
  const int cy = P.ny - 1;
  for (int j = blockIdx.x; j < B.nsteps; j += gridDim.x) {
    const StepShape r = build_step(P, B, j, X, L, s_sort, sh);
    if (r.rows == 0) { __syncthreads(); continue; }
    if (r.nv > B.vals_cap) {                               // the host sized vals from the counts
      if (threadIdx.x == 0) atomicOr(B.err, 1);
      __syncthreads();
      continue;
    }
    const int* U = X + L.u; const int* lo = X + L.lo; const int* row = X + L.row;
    const int* pv = X + L.pv; const int* po = X + L.po; const int* pl = X + L.pl; const int* ph = X + L.ph;
    // the vertices each owner pair evaluates, at consecutive value slots
    for (int pr = threadIdx.x; pr < 4 * r.nu; pr += kRThreads) {
      if (po[pr] != pr) continue;
      const int cc = U[pr >> 2], vi = cc / cy + ((pr & 3) >> 1), vj = cc % cy + (pr & 1);
      const int base = (int)((size_t)vi * P.ny + vj) * P.nz;
      for (int kk = pl[pr]; kk <= ph[pr]; ++kk) vpt[pv[pr] + (kk - pl[pr])] = base + kk;
    }
    __syncthreads();
    const int k = B.k0 + j;
    const int slot = k - W.base + 1;
    if (threadIdx.x == 0 && B.pairs)                  // the point x node pairs of both times
      atomicAdd(B.pairs, (unsigned long long)r.nv * (W.count[slot] + (k > 0 ? W.count[slot - 1] : 0)));
    eval_vertices<PREC>(P, W, slot, vpt, r.nv, Tc, (float4*)s_sort);
    if (k > 0) {
      eval_vertices<PREC>(P, W, slot - 1, vpt, r.nv, Tp, (float4*)s_sort);
    } else {
      for (int v = threadIdx.x; v < r.nv; v += kRThreads) Tp[v] = P.T0;
      __syncthreads();
    }
    const double t = W.t[slot];
    const double t_prev = t - P.dt;
    const long long rb = B.row_base[j];
    for (int q = threadIdx.x; q < r.rows; q += kRThreads) {
      int a = 0, b = r.nu - 1;                        // the cell column whose run holds row q
      while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (row[m] <= q) a = m; else b = m - 1;
      }
      const int u = a, ck = lo[u] + (q - row[u]);
      const int cc = U[u];
      const long long R = rb + q;
      B.idx[3 * R] = (uint32_t)(cc / cy);
      B.idx[3 * R + 1] = (uint32_t)(cc % cy);
      B.idx[3 * R + 2] = (uint32_t)ck;
      B.ts[2 * R] = t_prev;
      B.ts[2 * R + 1] = t;
      double* o = B.Ts + 16 * R;
#pragma unroll
      for (int nvx = 0; nvx < 8; ++nvx) {             // vertex (di, dj, dk), di slowest
        const int own = po[4 * u + (nvx >> 1)];
        const int vi = pv[own] + (ck + (nvx & 1) - pl[own]);
        o[nvx] = Tp[vi];
        o[8 + nvx] = Tc[vi];
      }
    }
    __syncthreads();
  }
}

}  // namespace

size_t th_rrdf_scratch_ints(int nmax) { return layout_for(nmax < 1 ? 1 : nmax).total; }

void th_launch_rrdf(const DevProblem& P, const NodeWindow& w, const RrdfBatch& b, bool fill, int precision, int blocks,
                    cudaStream_t s) {
  if (b.nsteps <= 0 || blocks <= 0) return;
  if (!fill) { k_rrdf_count<<<blocks, kRThreads, 0, s>>>(P, b); return; }
  if (precision == 0) k_rrdf_fill<0><<<blocks, kRThreads, 0, s>>>(P, w, b);
  else k_rrdf_fill<1><<<blocks, kRThreads, 0, s>>>(P, w, b);
}
