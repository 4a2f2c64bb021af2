// Device helpers shared by the temperature, tracking and solidification kernels.
#pragma once
#include <cstdint>

#include "th_kernels.h"
#include "th_nodes.cuh"

namespace thdev {

constexpr double kNeg3Log2e = -3.0 * 1.4426950408889634;   // -3 * log2(e)

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Grid coordinates recomputed from indices (src/Grid.h:310-327): min + i * ((max - min) / (n - 1)),
// or max on a single-point axis.  Rounded exactly as the reference rounds them.
// Packed FP32 pairs (sm_100+ f32x2 arithmetic): two points' values in one 64-bit register.
__device__ __forceinline__ unsigned long long pk2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long add2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long sub2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__device__ __forceinline__ double coord(int g, double vmin, double vmax, double h, int i) {
  return (g - 1) ? rn_add(vmin, rn_mul((double)i, h)) : vmax;
}

__device__ __forceinline__ void store_node(const NodeBufView& nb, int slot, const NodeVal& v) {
  nb.x[slot] = v.x; nb.y[slot] = v.y; nb.z[slot] = v.z;
  nb.ipx[slot] = v.ipx; nb.ipy[slot] = v.ipy; nb.ipz[slot] = v.ipz;
  nb.dtau[slot] = v.dtau; nb.amp[slot] = v.amp;
  nb.kx[slot] = __double2float_rn(kNeg3Log2e * v.ipx);
  nb.ky[slot] = __double2float_rn(kNeg3Log2e * v.ipy);
  nb.kz[slot] = __double2float_rn(kNeg3Log2e * v.ipz);
  nb.w[slot] = __double2float_rn(v.dtau * v.amp);
  const float xh = __double2float_rn(v.x), yh = __double2float_rn(v.y), zh = __double2float_rn(v.z);
  nb.xh[slot] = xh; nb.xl[slot] = __double2float_rn(v.x - (double)xh);
  nb.yh[slot] = yh; nb.yl[slot] = __double2float_rn(v.y - (double)yh);
  nb.zh[slot] = zh; nb.zl[slot] = __double2float_rn(v.z - (double)zh);
}

__device__ __forceinline__ void point_xyz(const DevProblem& P, int64_t p, double& x, double& y, double& z) {
  if (P.cx) {                               // custom points (Grid::get_x with its x array, src/Grid.h:310-327)
    x = P.cx[p]; y = P.cy[p]; z = P.cz[p];
    return;
  }
  const int64_t nyz = (int64_t)P.ny * P.nz;
  const int i = (int)(p / nyz), j = (int)((p / P.nz) % P.ny), k = (int)(p % P.nz);
  x = coord(P.gx, P.xmin, P.xmax, P.hx, i);
  y = coord(P.gy, P.ymin, P.ymax, P.hy, j);
  z = coord(P.gz, P.zmin, P.zmax, P.hz, k);
}

// One thread block builds the whole node list at time t (the reference's GaussIntegrate
// order: beams in order; per beam the zero-weight node at t, then the quadrature
// intervals in walk order, each interval's Gauss points from the late end).  Thread 0
// walks the path serially in exact FP64 (the interval schedule only needs a few FP64
// operations per interval) and fills a shared-memory chunk of up to kChunkIntervals
// intervals; then every thread builds candidate nodes of the chunk in parallel and a block
// scan compacts the kept ones in order.  Image copies for the boundary planes follow
// (src/Calc.cpp:584-605).  blockDim.x must be kGenThreads.
constexpr int kGenThreads = 256;
constexpr int kListPad = 128;         // node lists are padded with zero-weight nodes to a multiple of this
constexpr int kChunkIntervals = 256;
constexpr int kSegCache = 320;        // path segments staged in shared memory per beam

struct GenShared {
  DevSeg seg_cache[kSegCache];
  double t1[kChunkIntervals], t2[kChunkIntervals];
  int seg[kChunkIntervals], ord[kChunkIntervals], off[kChunkIntervals + 1];
  int wsum[kGenThreads / 32];
  int m, more, nout, err, kept;
};

// The combined intervals' centre and mean power of a chunk (path compression only); the
// kernels that generate lists take it as dynamic shared memory when the deck compresses.
struct GenComp {
  double cx[kChunkIntervals], cy[kChunkIntervals], cq[kChunkIntervals];
};
constexpr int kOrdComb = 0x100;        // flag in GenShared::ord: a combined interval

// Every beam's nodes appended to the list (sh.nout counts them, nodes past nb.cap are
// counted but not stored): the plain walk, or with cs the compressed walk.
__device__ __forceinline__ void gen_walk_block(const DevProblem& P, double t, bool is_sol, const NodeBufView& nb,
                                               GenShared& sh, GenComp* cs) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    if (B.nseg <= kSegCache) {                         // the walk touches every segment: stage them
      __syncthreads();
      for (int i = tid; i < B.nseg; i += kGenThreads) sh.seg_cache[i] = path[i];
      __syncthreads();
      path = sh.seg_cache;
    }
    Walk W;
    CWalk C;
    if (tid == 0) {
      NodeVal v;
      bool inst;
      if (cs) { cwalk_begin(B, path, t, is_sol, C); W.t = t; W.s = C.s; inst = instant_node(P, B, path, W, v); }
      else { walk_begin(B, path, t, is_sol, W); inst = instant_node(P, B, path, W, v); }
      if (inst) {
        if (sh.nout < nb.cap) store_node(nb, sh.nout, v);
        sh.nout++;
      }
    }
    int steps = 0;
    while (true) {
      __syncthreads();
      if (tid == 0) {                                  // next chunk of the interval schedule
        int m = 0, off = 0;
        if (cs) {
          CInterval I;
          while (m < kChunkIntervals) {
            if (++steps > kMaxWalkSteps) { sh.err |= ERR_WALK_LIMIT; C.more = false; break; }
            int e = 0;
            const bool got = cwalk_next(P, B, path, C, I, e);
            sh.err |= e;
            if (!got) break;
            sh.t1[m] = I.t1; sh.t2[m] = I.t2; sh.seg[m] = I.s; sh.ord[m] = I.order | (I.comb ? kOrdComb : 0);
            cs->cx[m] = I.cx; cs->cy[m] = I.cy; cs->cq[m] = I.cq;
            sh.off[m] = off;
            off += I.order;
            ++m;
            if (!C.more) break;
          }
          sh.more = C.more;
        } else {
          while (W.more && m < kChunkIntervals) {
            if (++steps > kMaxWalkSteps) { sh.err |= ERR_WALK_LIMIT; W.more = false; break; }
            walk_interval(B, path, W);
            sh.t1[m] = W.t1; sh.t2[m] = W.t2; sh.seg[m] = W.s; sh.ord[m] = W.order; sh.off[m] = off;
            off += W.order;
            ++m;
            walk_advance(W);
          }
          sh.more = W.more;
        }
        sh.off[m] = off;
        sh.m = m;
      }
      __syncthreads();
      const int m = sh.m, total = sh.off[m];
      for (int base = 0; base < total; base += kGenThreads) {
        const int c = base + tid;
        bool keep = false;
        NodeVal v;
        if (c < total) {
          int lo = 0, hi = m - 1;                      // interval of candidate c
          while (lo < hi) { const int mid = (lo + hi + 1) >> 1; if (sh.off[mid] <= c) lo = mid; else hi = mid - 1; }
          const int order = sh.ord[lo] & 0xff, g = c - sh.off[lo];
          const int k = order - 2 + order - 1 - g;
          if (sh.ord[lo] & kOrdComb) {
            CInterval I;
            I.t1 = sh.t1[lo]; I.t2 = sh.t2[lo]; I.s = sh.seg[lo]; I.order = order; I.comb = true;
            I.cx = cs->cx[lo]; I.cy = cs->cy[lo]; I.cq = cs->cq[lo];
            keep = comb_node(P, B, path, I, t, k, g, v);
          } else {
            Walk w;
            w.t = t; w.t1 = sh.t1[lo]; w.t2 = sh.t2[lo]; w.s = sh.seg[lo];
            keep = gauss_node(P, B, path, w, k, v);
          }
        }
        const unsigned mk = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) sh.wsum[warp] = __popc(mk);
        __syncthreads();
        if (tid == 0) {
          int acc = 0;
          for (int i = 0; i < kGenThreads / 32; ++i) { const int x = sh.wsum[i]; sh.wsum[i] = acc; acc += x; }
          sh.kept = acc;
        }
        __syncthreads();
        const int slot = sh.nout + sh.wsum[warp] + __popc(mk & ((1u << lane) - 1u));
        if (keep && slot < nb.cap) store_node(nb, slot, v);
        __syncthreads();
        if (tid == 0) sh.nout += sh.kept;
        __syncthreads();
      }
      if (!sh.more) break;
    }
  }
}

__device__ __forceinline__ void copy_node(const NodeBufView& nb, int dst, int src) {
  nb.x[dst] = nb.x[src]; nb.y[dst] = nb.y[src]; nb.z[dst] = nb.z[src];
  nb.ipx[dst] = nb.ipx[src]; nb.ipy[dst] = nb.ipy[src]; nb.ipz[dst] = nb.ipz[src];
  nb.dtau[dst] = nb.dtau[src]; nb.amp[dst] = nb.amp[src];
  nb.kx[dst] = nb.kx[src]; nb.ky[dst] = nb.ky[src]; nb.kz[dst] = nb.kz[src]; nb.w[dst] = nb.w[src];
  nb.xh[dst] = nb.xh[src]; nb.xl[dst] = nb.xl[src]; nb.yh[dst] = nb.yh[src]; nb.yl[dst] = nb.yl[src];
  nb.zh[dst] = nb.zh[src]; nb.zl[dst] = nb.zl[src];
}

// One thread block builds the whole node list at time t (Calc::Integrate_Serial,
// src/Calc.cpp:48-65).  With path compression (P.compress; cs must then point at the
// block's GenComp) the list is the compressed walk's, except at a non-solidification time
// where the plain walk's list is kept when it is not longer (the reference builds both and
// keeps the smaller, src/Calc.cpp:49-58): both are built, the plain one after the
// compressed one, so the buffer must hold both (a count above nb.cap reports the need).
__device__ __forceinline__ void gen_list_block(const DevProblem& P, double t, bool is_sol, const NodeBufView& nb,
                                               int* count, int* err, GenShared& sh, GenComp* cs = nullptr) {
  const int tid = threadIdx.x;
  if (tid == 0) { sh.nout = 0; sh.err = 0; }
  __syncthreads();
  if (P.compress && cs) {
    gen_walk_block(P, t, is_sol, nb, sh, cs);
    if (!is_sol) {
      __syncthreads();
      const int n_c = sh.nout;
      gen_walk_block(P, t, is_sol, nb, sh, nullptr);
      __syncthreads();
      const int n_r = sh.nout - n_c;
      if (sh.nout <= nb.cap) {
        if (n_r <= n_c) {                              // keep the plain list: move it down
          for (int i = tid; i < n_r; i += kGenThreads) copy_node(nb, i, n_c + i);
          __syncthreads();
          if (tid == 0) sh.nout = n_r;
        } else if (tid == 0) {
          sh.nout = n_c;
        }
      }
      __syncthreads();
    }
  } else {
    if (P.compress && tid == 0) sh.err |= ERR_WALK_LIMIT;   // a compressing deck needs cs
    gen_walk_block(P, t, is_sol, nb, sh, nullptr);
  }
  __syncthreads();
  const int n0 = sh.nout;
  int n = n0;
  if (P.n_images > 1) {
    if ((long long)n0 * P.n_images > nb.cap) {
      if (tid == 0) sh.err |= ERR_NODE_CAPACITY;
    } else {
      for (int idx = tid; idx < n0 * (P.n_images - 1); idx += kGenThreads) {
        const int im = 1 + idx / n0, j = idx % n0;
        NodeVal v;
        v.x = image_coord(P.img[im][0], P.bcx0, P.bcx1, nb.x[j]);
        v.y = image_coord(P.img[im][1], P.bcy0, P.bcy1, nb.y[j]);
        v.z = image_coord(P.img[im][2], P.bcz0, P.bcz1, nb.z[j]);
        v.ipx = nb.ipx[j]; v.ipy = nb.ipy[j]; v.ipz = nb.ipz[j]; v.dtau = nb.dtau[j]; v.amp = nb.amp[j];
        store_node(nb, im * n0 + j, v);
      }
    }
    n = n0 * P.n_images;
  }
  // zero-weight nodes up to a multiple of kListPad (they add exactly nothing), so that the
  // FP32 tracking passes give every lane of a warp the same number of four-node groups
  if (n <= nb.cap)
    for (int s = n + tid; s < ((n + kListPad - 1) & ~(kListPad - 1)) && s < nb.cap; s += kGenThreads)
      store_node(nb, s, NodeVal{});
  __syncthreads();
  if (tid == 0) {
    int e = sh.err;
    if (n > nb.cap) e |= ERR_NODE_CAPACITY;
    *count = n;
    if (e) atomicOr(err, e);
  }
}

}  // namespace thdev
