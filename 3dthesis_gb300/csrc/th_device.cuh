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
  const int64_t nyz = (int64_t)P.ny * P.nz;
  const int i = (int)(p / nyz), j = (int)((p / P.nz) % P.ny), k = (int)(p % P.nz);
  x = coord(P.gx, P.xmin, P.xmax, P.hx, i);
  y = coord(P.gy, P.ymin, P.ymax, P.hy, j);
  z = coord(P.gz, P.zmin, P.zmax, P.hz, k);
}

// One warp builds the whole node list at time t: beams in order, each beam's intervals in
// walk order, the Gauss points of an interval spread over the lanes (lane l takes the
// l-th point from the late end, the reference's emission order), kept nodes compacted
// with a ballot.  Image copies for the boundary planes follow (src/Calc.cpp:584-605).
__device__ __forceinline__ void gen_list_warp(const DevProblem& P, double t, bool is_sol, const NodeBufView& nb,
                                              int* count, int* err) {
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  int n = 0;
  int e = 0;
  for (int b = 0; b < P.nbeams; ++b) {
    const DevBeam B = P.beam[b];
    const DevSeg* path = P.segs + B.seg_off;
    Walk W;
    walk_begin(B, path, t, is_sol, W);
    {
      NodeVal v;
      const bool keep = instant_node(P, B, path, W, v);
      if (keep) {
        if (lane == 0 && n < nb.cap) store_node(nb, n, v);
        ++n;
      }
    }
    int steps = 0;
    while (W.more) {
      if (++steps > kMaxWalkSteps) { e |= ERR_WALK_LIMIT; break; }
      walk_interval(B, path, W);
      const int base = W.order - 2;
      NodeVal v;
      bool keep = false;
      if (lane < W.order) keep = gauss_node(P, B, path, W, base + W.order - 1 - lane, v);
      const unsigned m = __ballot_sync(full, keep);
      const int slot = n + __popc(m & ((1u << lane) - 1u));
      if (keep && slot < nb.cap) store_node(nb, slot, v);
      n += __popc(m);
      walk_advance(W);
    }
  }
  const int n0 = n;
  if (P.n_images > 1) {
    if ((long long)n0 * P.n_images > nb.cap) {
      e |= ERR_NODE_CAPACITY;
    } else {
      __syncwarp();
      for (int im = 1; im < P.n_images; ++im) {
        for (int j = lane; j < n0; j += 32) {
          NodeVal v;
          v.x = image_coord(P.img[im][0], P.bcx0, P.bcx1, nb.x[j]);
          v.y = image_coord(P.img[im][1], P.bcy0, P.bcy1, nb.y[j]);
          v.z = image_coord(P.img[im][2], P.bcz0, P.bcz1, nb.z[j]);
          v.ipx = nb.ipx[j]; v.ipy = nb.ipy[j]; v.ipz = nb.ipz[j]; v.dtau = nb.dtau[j]; v.amp = nb.amp[j];
          store_node(nb, im * n0 + j, v);
        }
      }
    }
    n = n0 * P.n_images;
  }
  if (n > nb.cap) e |= ERR_NODE_CAPACITY;
  if (lane == 0) {
    *count = n;
    if (e) atomicOr(err, e);
  }
}

}  // namespace thdev
