// Device-side quadrature-node generation (the reference's Calc::GaussIntegrate,
// src/Calc.cpp:67-211, with Util::GetBeamLoc / GetRefTime / InRMax / AddToNodes,
// src/Util.cpp:40-50,168-237).
//
// Every floating-point step uses the explicitly rounded double intrinsics (__dadd_rn,
// __dmul_rn, ...) in the reference's operation order, so no multiply-add is contracted
// and the node times, positions, weights and the keep/drop decisions are bit-identical
// to the reference's double-precision host code.  The only departure is the node
// amplitude: the reference stores expmod = log(q beta) - log(phix phiy phiz)/2 and
// later evaluates exp(... + expmod); this code stores amp = q beta / sqrt(phix phiy phiz)
// directly and multiplies, which avoids two logs per node and agrees to a few ulps.
#pragma once
#include "th_problem.h"

namespace thdev {

__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double rn_sqrt(double a) { return __dsqrt_rn(a); }

// Upper bound on walk iterations per beam; a deck that needs more reports an error
// instead of looping (a zero width or speed would otherwise never advance).
constexpr int kMaxWalkSteps = 1 << 20;

enum { ERR_NODE_CAPACITY = 1, ERR_WALK_LIMIT = 2, ERR_LIST_CAPACITY = 4, ERR_ROUND_LIMIT = 8 };

struct BeamLoc { double x, y, z, q; };

// Beam position at time t on segment s (src/Util.cpp:211-237): a spot sits at the
// segment end; a line interpolates between the previous and current end points.
// Power is zeroed outside the domain grown by r_max (src/Util.cpp:168-172).
__device__ __forceinline__ BeamLoc beam_loc(const DevProblem& P, const DevSeg* path, double t, int s) {
  const DevSeg cur = path[s];
  BeamLoc L;
  if (cur.mode) {
    L.x = cur.x; L.y = cur.y; L.z = cur.z;
  } else {
    const DevSeg prv = path[s - 1];
    const double r = rn_div(rn_sub(t, prv.tend), rn_sub(cur.tend, prv.tend));
    L.x = rn_add(prv.x, rn_mul(r, rn_sub(cur.x, prv.x)));
    L.y = rn_add(prv.y, rn_mul(r, rn_sub(cur.y, prv.y)));
    L.z = rn_add(prv.z, rn_mul(r, rn_sub(cur.z, prv.z)));
  }
  const bool out = (L.x > P.rx1) || (L.x < P.rx0) || (L.y > P.ry1) || (L.y < P.ry0);
  L.q = out ? 0.0 : cur.q;
  return L;
}

// Largest quadrature step allowed on segment s after tpp seconds of look-back
// (src/Util.cpp:192-209).
__device__ __forceinline__ double ref_time(const DevBeam& B, const DevSeg* path, double tpp, int s) {
  double spp = rn_div(tpp, B.nond);
  spp = (spp < 0.0) ? 0.0 : spp;
  if (path[s].mode == 0) return rn_mul(path[s].rt0, rn_sqrt(rn_add(rn_mul(12.0, spp), 1.0)));
  double r = rn_sub(path[s].tend, path[s - 1].tend);
  if (r == 0) r = 1.0e-9;
  return r;
}

// First segment s >= 1 whose end time is not before t, clamped to the last segment:
// the segment the reference's upward search from segment 1 lands on (src/Calc.cpp:99).
__device__ __forceinline__ int find_seg(const DevSeg* path, int nseg, double t) {
  int lo = 1, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (t > path[mid].tend) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// State of the backward walk along one beam's path.
struct Walk {
  double t, t1, t2, tpp, stepmax, step0;
  int s, order;
  bool more, sw;
};

__device__ __forceinline__ void walk_begin(const DevBeam& B, const DevSeg* path, double t, bool is_sol, Walk& W) {
  W.t = t;
  W.s = find_seg(path, B.nseg, t);
  W.step0 = is_sol ? rn_mul(B.nond, B.az) : B.nond;
  W.stepmax = W.step0;
  W.order = 16;
  W.t2 = t; W.t1 = t; W.tpp = 0.0;
  if (t > B.tlast) { W.tpp = rn_add(W.tpp, rn_sub(t, B.tlast)); W.t2 = B.tlast; }
  int guard = 0;
  while (W.tpp >= rn_sub(rn_mul(2.0, W.stepmax), W.step0) && guard++ < 4096) {
    W.stepmax = rn_mul(W.stepmax, 2.0);
    if (W.order != 2) W.order /= 2;
  }
  W.more = true;
  W.sw = false;
}

// Next quadrature interval [t1, t2] on segment s; clips at the segment start and marks
// the segment switch, or the end of the walk at t = 0 (src/Calc.cpp:151-173).
__device__ __forceinline__ void walk_interval(const DevBeam& B, const DevSeg* path, Walk& W) {
  const double rt = ref_time(B, path, W.tpp, W.s);
  const double use = (rt < W.stepmax) ? rt : W.stepmax;
  W.t1 = rn_sub(W.t2, use);
  const double next = path[W.s - 1].tend;
  W.sw = false;
  if (W.t1 <= next) {
    W.t1 = next;
    if (next > 0.0) W.sw = true; else W.more = false;
  }
}

// Step bookkeeping after the interval's nodes are emitted (src/Calc.cpp:192-207).
__device__ __forceinline__ void walk_advance(Walk& W) {
  if (W.sw) W.s--;
  W.tpp = rn_add(W.tpp, rn_sub(W.t2, W.t1));
  W.t2 = W.t1;
  if (W.tpp >= rn_sub(rn_mul(2.0, W.stepmax), W.step0)) {
    W.stepmax = rn_mul(W.stepmax, 2.0);
    if (W.order != 2) W.order /= 2;
  }
}

struct NodeVal {
  double x, y, z, ipx, ipy, ipz, dtau, amp;
};

__device__ __forceinline__ void finish_node(const DevBeam& B, double ct, double qb, double dtau, const BeamLoc& L, NodeVal& v) {
  const double phx = rn_add(B.ax2, ct), phy = rn_add(B.ay2, ct), phz = rn_add(B.az2, ct);
  v.x = L.x; v.y = L.y; v.z = L.z;
  v.ipx = rn_div(1.0, phx); v.ipy = rn_div(1.0, phy); v.ipz = rn_div(1.0, phz);
  v.dtau = dtau;
  v.amp = rn_div(qb, rn_sqrt(rn_mul(rn_mul(phx, phy), phz)));
}

// Node k (absolute index into the packed Gauss tables) of the current interval; returns
// whether the reference keeps it (q beta > 0 and dtau > 0; src/Calc.cpp:176-190).
__device__ __forceinline__ bool gauss_node(const DevProblem& P, const DevBeam& B, const DevSeg* path, const Walk& W,
                                           int k, NodeVal& v) {
  const double h = rn_sub(W.t2, W.t1);
  const double tp = rn_mul(0.5, rn_add(rn_mul(h, P.gl_loc[k]), rn_add(W.t2, W.t1)));
  const double ct = rn_mul(P.a12, rn_sub(W.t, tp));
  const BeamLoc L = beam_loc(P, path, tp, W.s);
  const double qb = rn_mul(L.q, B.beta);
  const double dtau = rn_mul(rn_mul(0.5, h), P.gl_w[k]);
  if (!(qb > 0.0 && dtau > 0.0)) return false;
  finish_node(B, ct, qb, dtau, L, v);
  return true;
}

// The zero-weight node at the current beam position, kept for the instantaneous source
// term of dT/dt (src/Calc.cpp:124-132).
__device__ __forceinline__ bool instant_node(const DevProblem& P, const DevBeam& B, const DevSeg* path, const Walk& W,
                                             NodeVal& v) {
  const BeamLoc L = beam_loc(P, path, W.t, W.s);
  const double qb = rn_mul(L.q, B.beta);
  if (!(W.t <= B.tlast && qb > 0.0)) return false;
  finish_node(B, 0.0, qb, 0.0, L, v);
  return true;
}

// Method-of-images copy of a coordinate (src/Calc.cpp:588-603).
__device__ __forceinline__ double image_coord(int c, double lo, double hi, double v) {
  const int n = abs(c % 2);
  return rn_add(rn_sub(rn_mul((double)(c + n), hi), rn_mul((double)(c - n), lo)), rn_mul((double)(1 - 2 * n), v));
}

}  // namespace thdev
