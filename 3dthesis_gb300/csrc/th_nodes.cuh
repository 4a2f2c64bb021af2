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

// ---------------------------------------------------------------- path compression
// The walk of Calc::GaussCompressIntegrate (src/Calc.cpp:213-501): like the plain walk,
// except that where an interval would reach into the previous segment, the segments whose
// end points lie within the heat's diffusion distance r of the beam position at t2
// (r^2 = ln2/8 ax^2 (12 a (t - t2) / ax^2 + 1)) and whose power matches are combined into
// one interval whose Gauss nodes all sit at the power-and-time weighted centre of the
// combined stretch, with its mean power.  Restated in the reference's operation order; the
// combined nodes' power takes one more factor beta per node (src/Calc.cpp:453-464), and
// their z - never set by the reference, an uninitialised int_seg (src/Calc.cpp:433), 0 in its
// builds on paths at z = 0 - is the z of the segment the interval starts from.  A segment
// end outside the r_max box, on which the reference's skip loop spins forever
// (src/Calc.cpp:303-316), ends the walk with ERR_WALK_LIMIT.
struct CWalk {
  double t, t2, tpp, stepmax, step0;
  int s, order;
  bool more;
};

// One interval of the compressed walk: [t1, t2], its Gauss order, the segment whose beam
// position gives its nodes (comb = false) or the combined centre and mean power (comb).
struct CInterval {
  double t1, t2, cx, cy, cq;
  int s, order;
  bool comb;
};

constexpr double kLn2 = 0.6931471805599453;    // ln 2, the double nearest to it

__device__ __forceinline__ bool in_rmax(const DevProblem& P, double x, double y) {
  return !((x > P.rx1) || (x < P.rx0) || (y > P.ry1) || (y < P.ry0));
}

static __device__ __noinline__ void cwalk_begin(const DevBeam& B, const DevSeg* path, double t, bool is_sol, CWalk& W) {
  W.t = t;
  W.s = find_seg(path, B.nseg, t);
  W.step0 = is_sol ? rn_mul(B.nond, B.az) : B.nond;
  W.stepmax = W.step0;
  W.order = 16;
  W.t2 = t; W.tpp = 0.0;
  if (t > B.tlast) { W.tpp = rn_add(W.tpp, rn_sub(t, B.tlast)); W.t2 = B.tlast; }
  int guard = 0;
  while (W.tpp >= rn_sub(rn_mul(2.0, W.stepmax), W.step0) && guard++ < 4096) {
    W.stepmax = rn_mul(W.stepmax, 2.0);
    if (W.order != 2) W.order /= 2;
  }
  W.more = true;
}

// The next interval of the compressed walk into I; false when the walk has ended without
// one.  err receives ERR_WALK_LIMIT for a segment end outside the r_max box.
static __device__ __noinline__ bool cwalk_next(const DevProblem& P, const DevBeam& B, const DevSeg* path, CWalk& W,
                                           CInterval& I, int& err) {
  if (!W.more) return false;
  if (path[W.s].tend <= 0.0) { W.more = false; return false; }
  if (!in_rmax(P, path[W.s].x, path[W.s].y)) { err |= ERR_WALK_LIMIT; W.more = false; return false; }
  int guard = 0;
  while (W.tpp >= rn_sub(rn_mul(2.0, W.stepmax), W.step0) && guard++ < 4096) {
    W.stepmax = rn_mul(W.stepmax, 2.0);
    if (W.order != 2) W.order /= 2;
  }
  const double rt = ref_time(B, path, W.tpp, W.s);
  const double use = (rt < W.stepmax) ? rt : W.stepmax;
  const BeamLoc Lp = beam_loc(P, path, W.t2, W.s);
  const double xp = Lp.x, yp = Lp.y;
  const double r2 = rn_mul(rn_mul(kLn2 / 8.0, B.ax2),
                           rn_add(rn_div(rn_mul(rn_mul(12.0, rn_sub(W.t, W.t2)), P.a), B.ax2), 1.0));
  int s2 = W.s, ncomb = 0;
  double t1 = path[W.s - 1].tend;
  double sum_t = 0.0, sum_qt = 0.0, sum_qtx = 0.0, sum_qty = 0.0;
  if (t1 < rn_sub(W.t2, use)) {
    t1 = rn_sub(W.t2, use);
  } else {
    for (int it = 0;; ++it) {                              // combine segments (src/Calc.cpp:350-425)
      if (it > kMaxWalkSteps) { err |= ERR_WALK_LIMIT; W.more = false; break; }
      if (path[s2 - 1].tend <= 0.0) { W.more = false; break; }
      double xs = path[s2 - 1].x, ys = path[s2 - 1].y;
      const double dist2 = rn_add(rn_mul(rn_sub(xs, xp), rn_sub(xs, xp)), rn_mul(rn_sub(ys, yp), rn_sub(ys, yp)));
      const double ts = path[s2 - 1].tend;
      if (!in_rmax(P, xp, yp)) break;
      const DevSeg cur = path[s2], prv = path[s2 - 1];
      bool stop = false;
      if ((dist2 > r2) ||
          (cur.q != prv.q && (W.order > 2 || rn_sub(W.t2, ts) > rn_div(W.stepmax, 64.0)))) {
        if (cur.mode) {
          const double d = rn_sub(t1, ts);
          sum_qtx = rn_add(sum_qtx, rn_mul(rn_mul(cur.x, cur.q), d));
          sum_qty = rn_add(sum_qty, rn_mul(rn_mul(cur.y, cur.q), d));
          sum_qt = rn_add(sum_qt, rn_mul(cur.q, d));
          sum_t = rn_add(sum_t, d);
          t1 = ts;
        } else {
          const double dx = rn_sub(cur.x, prv.x), dy = rn_sub(cur.y, prv.y), dt = rn_sub(cur.tend, ts);
          const double den = rn_add(rn_mul(dx, dx), rn_mul(dy, dy));
          const double num = rn_add(rn_mul(rn_sub(xp, xs), rn_sub(xp, xs)), rn_mul(rn_sub(yp, ys), rn_sub(yp, ys)));
          double t_int = rn_add(ts, rn_mul(dt, rn_sub(rn_sqrt(rn_div(num, den)), rn_sqrt(rn_div(r2, den)))));
          if (t_int < rn_sub(W.t2, W.stepmax)) t_int = rn_sub(W.t2, W.stepmax);
          const double mid = rn_sub(rn_div(rn_add(t1, t_int), 2.0), ts);
          const double px = rn_add(xs, rn_div(rn_mul(dx, mid), dt)), py = rn_add(ys, rn_div(rn_mul(dy, mid), dt));
          const double d = rn_sub(t1, t_int);
          sum_qtx = rn_add(sum_qtx, rn_mul(rn_mul(px, cur.q), d));
          sum_qty = rn_add(sum_qty, rn_mul(rn_mul(py, cur.q), d));
          sum_qt = rn_add(sum_qt, rn_mul(cur.q, d));
          sum_t = rn_add(sum_t, d);
          t1 = t_int;
        }
        stop = true;
      } else {
        if (ts < rn_sub(W.t2, W.stepmax)) { stop = true; t1 = rn_sub(W.t2, W.stepmax); }
        else { t1 = ts; ++ncomb; }
        const double dt = rn_sub(cur.tend, t1);
        if (cur.mode) {
          sum_qtx = rn_add(sum_qtx, rn_mul(rn_mul(cur.x, cur.q), dt));
          sum_qty = rn_add(sum_qty, rn_mul(rn_mul(cur.y, cur.q), dt));
        } else {
          const double dx = rn_sub(cur.x, prv.x), dy = rn_sub(cur.y, prv.y);
          const double mid = rn_sub(rn_div(rn_add(cur.tend, t1), 2.0), ts);
          sum_qtx = rn_add(sum_qtx, rn_mul(rn_mul(rn_add(xs, rn_div(rn_mul(dx, mid), dt)), cur.q), dt));
          sum_qty = rn_add(sum_qty, rn_mul(rn_mul(rn_add(ys, rn_div(rn_mul(dy, mid), dt)), cur.q), dt));
        }
        sum_qt = rn_add(sum_qt, rn_mul(cur.q, dt));
        sum_t = rn_add(sum_t, dt);
      }
      if (t1 == path[s2 - 1].tend) {
        xs = path[s2 - 1].x;
        ys = path[s2 - 1].y;
        --s2;
        if (!in_rmax(P, xs, ys)) break;
      }
      if (stop) break;
    }
    if (!ncomb) { t1 = path[W.s - 1].tend; s2 = W.s - 1; }
  }
  I.t1 = t1; I.t2 = W.t2; I.s = W.s; I.order = W.order; I.comb = ncomb != 0;
  I.cx = I.cy = I.cq = 0.0;
  if (I.comb && sum_qt > 0.0) {
    I.cx = rn_div(sum_qtx, sum_qt);
    I.cy = rn_div(sum_qty, sum_qt);
    I.cq = rn_div(sum_qt, sum_t);
  }
  W.tpp = rn_add(W.tpp, rn_sub(W.t2, t1));
  W.t2 = t1;
  if (W.tpp >= rn_sub(rn_mul(2.0, W.stepmax), W.step0)) {
    W.stepmax = rn_mul(W.stepmax, 2.0);
    if (W.order != 2) W.order /= 2;
  }
  W.s = s2;
  if (t1 <= 0.0) W.more = false;
  return true;
}

// Node k (absolute index into the packed Gauss tables) of a combined interval, emitted j-th
// (0-based) in the interval's node order: at the combined centre, with the mean power times
// beta^(j+1) (the reference multiplies by beta once per emitted node).
static __device__ __noinline__ bool comb_node(const DevProblem& P, const DevBeam& B, const DevSeg* path,
                                          const CInterval& I, double t, int k, int j, NodeVal& v) {
  const double h = rn_sub(I.t2, I.t1);
  const double tp = rn_mul(0.5, rn_add(rn_mul(h, P.gl_loc[k]), rn_add(I.t2, I.t1)));
  const double ct = rn_mul(P.a12, rn_sub(t, tp));
  double q = I.cq;
  for (int i = 0; i <= j; ++i) q = rn_mul(q, B.beta);
  const double dtau = rn_mul(rn_mul(0.5, h), P.gl_w[k]);
  if (!(q > 0.0 && dtau > 0.0)) return false;
  BeamLoc L;
  L.x = I.cx; L.y = I.cy; L.z = path[I.s].z; L.q = q;
  finish_node(B, ct, q, dtau, L, v);
  return true;
}

// Method-of-images copy of a coordinate (src/Calc.cpp:588-603).
__device__ __forceinline__ double image_coord(int c, double lo, double hi, double v) {
  const int n = abs(c % 2);
  return rn_add(rn_sub(rn_mul((double)(c + n), hi), rn_mul((double)(c - n), lo)), rn_mul((double)(1 - 2 * n), v));
}

}  // namespace thdev
