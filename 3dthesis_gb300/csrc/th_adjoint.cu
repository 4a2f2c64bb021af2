// Adjoint of probe temperatures for calibration: dL/d{P, eta, Width_X, Width_Y, Depth_Z,
// alpha} and dL/d(path vertex x, y) of a single-beam problem, for a loss L of the
// temperatures at probe points and times.
//
// The node list is a function of the parameters through the quadrature walk: node times,
// weights and positions move with the widths, the diffusivity and the segment end times
// (which follow the vertices through the segment lengths).  The host re-walks the path in
// FP64 with the same operations in the same order as the device walk (src/Calc.cpp:67-211,
// src/Util.cpp:192-237), so the values are the device's node list bit for bit, while
// recording the walk for differentiation.  The device kernel recomputes every probe x node
// term (no pair storage) and sums, per node, the loss gradient with respect to the node's
// position, inverse widths and weight; a reverse sweep over the recorded walk carries those
// to every parameter at once.  (A forward-mode walk in dual numbers gives the node tangents
// themselves, for inspection.)  Discrete choices of the walk (interval counts, Gauss orders,
// the r_max cut-off) are held fixed, as a finite difference that does not cross one sees.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/thesis_gb300.h"
#include "th_device.cuh"
#include "th_kernels.h"
#include "th_problem.h"

using namespace thdev;

namespace {

// ------------------------------------------------------------------ forward mode
// Value and gradient over the parameter vector; an empty gradient is a constant.
struct Dual {
  double v = 0.0;
  std::vector<double> d;
  Dual() = default;
  Dual(double x) : v(x) {}
};

// r.d = a * x.d + b * y.d, treating an empty gradient as zero
void combine(Dual& r, double a, const Dual& x, double b, const Dual& y) {
  if (x.d.empty() && y.d.empty()) return;
  const size_t n = std::max(x.d.size(), y.d.size());
  r.d.assign(n, 0.0);
  if (!x.d.empty()) for (size_t i = 0; i < n; ++i) r.d[i] += a * x.d[i];
  if (!y.d.empty()) for (size_t i = 0; i < n; ++i) r.d[i] += b * y.d[i];
}

Dual operator+(const Dual& x, const Dual& y) { Dual r(x.v + y.v); combine(r, 1.0, x, 1.0, y); return r; }
Dual operator-(const Dual& x, const Dual& y) { Dual r(x.v - y.v); combine(r, 1.0, x, -1.0, y); return r; }
Dual operator*(const Dual& x, const Dual& y) { Dual r(x.v * y.v); combine(r, y.v, x, x.v, y); return r; }
Dual operator/(const Dual& x, const Dual& y) {
  Dual r(x.v / y.v);
  combine(r, 1.0 / y.v, x, -x.v / (y.v * y.v), y);
  return r;
}
// sqrt with a zero derivative at 0 (a zero-length segment, whose length is not
// differentiable there)
Dual dsqrt(const Dual& x) {
  Dual r(std::sqrt(x.v));
  combine(r, r.v > 0.0 ? 0.5 / r.v : 0.0, x, 0.0, Dual());
  return r;
}

// ------------------------------------------------------------------ reverse mode
// A value recorded on the tape: entry i has up to two parents with their partial
// derivatives; the first np entries are the parameters.  i < 0 is a constant.
struct TapeEntry { int a, b; double da, db; };
thread_local std::vector<TapeEntry>* g_tape = nullptr;

struct Rev {
  double v = 0.0;
  int i = -1;
  Rev() = default;
  Rev(double x) : v(x) {}
};

Rev record(double v, const Rev& x, double dx, const Rev& y, double dy) {
  Rev r(v);
  if (x.i < 0 && y.i < 0) return r;
  r.i = (int)g_tape->size();
  g_tape->push_back({x.i, y.i, dx, dy});
  return r;
}
Rev operator+(const Rev& x, const Rev& y) { return record(x.v + y.v, x, 1.0, y, 1.0); }
Rev operator-(const Rev& x, const Rev& y) { return record(x.v - y.v, x, 1.0, y, -1.0); }
Rev operator*(const Rev& x, const Rev& y) { return record(x.v * y.v, x, y.v, y, x.v); }
Rev operator/(const Rev& x, const Rev& y) { return record(x.v / y.v, x, 1.0 / y.v, y, -(x.v / y.v) / y.v); }
Rev dsqrt(const Rev& x) {
  const double s = std::sqrt(x.v);
  return record(s, x, s > 0.0 ? 0.5 / s : 0.0, Rev(), 0.0);
}

// ------------------------------------------------------------------ the walk, on either
template <class N> struct DSeg { N x, y, z, tend, rt0; double q, prm; int mode; };
template <class N> struct DBeam { N az, ax2, ay2, az2, nond, beta, tlast, a12; int nseg; };
template <class N> struct DNode { N x, y, z, ipx, ipy, ipz, dtau, amp; };
template <class N> struct DLoc { N x, y, z; double q; };

// src/Util.cpp:192-209
template <class N>
N ref_time(const DBeam<N>& B, const std::vector<DSeg<N>>& path, const N& tpp, int s) {
  N spp = tpp / B.nond;
  if (spp.v < 0.0) spp = N(0.0);
  if (path[s].mode == 0) return path[s].rt0 * dsqrt(N(12.0) * spp + N(1.0));
  N r = path[s].tend - path[s - 1].tend;
  if (r.v == 0) r = N(1.0e-9);
  return r;
}

template <class N>
int find_seg(const std::vector<DSeg<N>>& path, double t) {
  int lo = 1, hi = (int)path.size() - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (t > path[mid].tend.v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// src/Util.cpp:211-237 with the r_max cut-off of src/Util.cpp:168-172
template <class N>
DLoc<N> beam_loc(const DevProblem& P, const std::vector<DSeg<N>>& path, const N& t, int s) {
  const DSeg<N>& cur = path[s];
  DLoc<N> L;
  if (cur.mode) {
    L.x = cur.x; L.y = cur.y; L.z = cur.z;
  } else {
    const DSeg<N>& prv = path[s - 1];
    const N r = (t - prv.tend) / (cur.tend - prv.tend);
    L.x = prv.x + r * (cur.x - prv.x);
    L.y = prv.y + r * (cur.y - prv.y);
    L.z = prv.z + r * (cur.z - prv.z);
  }
  const bool out = (L.x.v > P.rx1) || (L.x.v < P.rx0) || (L.y.v > P.ry1) || (L.y.v < P.ry0);
  L.q = out ? 0.0 : cur.q;
  return L;
}

template <class N>
DNode<N> finish_node(const DBeam<N>& B, const N& ct, const N& qb, const N& dtau, const DLoc<N>& L) {
  const N phx = B.ax2 + ct, phy = B.ay2 + ct, phz = B.az2 + ct;
  DNode<N> v;
  v.x = L.x; v.y = L.y; v.z = L.z;
  v.ipx = N(1.0) / phx; v.ipy = N(1.0) / phy; v.ipz = N(1.0) / phz;
  v.dtau = dtau;
  v.amp = qb / dsqrt((phx * phy) * phz);
  return v;
}

// The node list at t in the device's order (zero-weight node, then each interval's Gauss
// points from the late end); returns false when the walk exceeds its step limit.
template <class N>
bool walk_nodes(const DevProblem& P, const DBeam<N>& B, const std::vector<DSeg<N>>& path, double t, bool is_sol,
                std::vector<DNode<N>>& out) {
  N t1, t2, tpp, stepmax, step0;
  int s = find_seg(path, t), order = 16;
  step0 = is_sol ? B.nond * B.az : B.nond;
  stepmax = step0;
  t2 = N(t); t1 = N(t); tpp = N(0.0);
  if (t > B.tlast.v) { tpp = tpp + (N(t) - B.tlast); t2 = B.tlast; }
  int guard = 0;
  while (tpp.v >= (N(2.0) * stepmax - step0).v && guard++ < 4096) {
    stepmax = stepmax * N(2.0);
    if (order != 2) order /= 2;
  }
  bool more = true, sw = false;
  {  // src/Calc.cpp:124-132
    const DLoc<N> L = beam_loc(P, path, N(t), s);
    if (t <= B.tlast.v && L.q * B.beta.v > 0.0) out.push_back(finish_node(B, N(0.0), N(L.q) * B.beta, N(0.0), L));
  }
  int steps = 0;
  while (more) {
    if (++steps > kMaxWalkSteps) return false;
    const N rt = ref_time(B, path, tpp, s);
    const N use = (rt.v < stepmax.v) ? rt : stepmax;
    t1 = t2 - use;
    const N next = path[s - 1].tend;
    sw = false;
    if (t1.v <= next.v) {
      t1 = next;
      if (next.v > 0.0) sw = true; else more = false;
    }
    const int base = order - 2;
    for (int k = base + order - 1; k >= base; --k) {         // src/Calc.cpp:176-190
      const N h = t2 - t1;
      const N tp = N(0.5) * ((h * N(P.gl_loc[k])) + (t2 + t1));
      const N ct = B.a12 * (N(t) - tp);
      const DLoc<N> L = beam_loc(P, path, tp, s);
      const N qb = N(L.q) * B.beta;
      const N dtau = (N(0.5) * h) * N(P.gl_w[k]);
      if (!(qb.v > 0.0 && dtau.v > 0.0)) continue;
      out.push_back(finish_node(B, ct, qb, dtau, L));
    }
    if (sw) s--;                                              // src/Calc.cpp:192-207
    tpp = tpp + (t2 - t1);
    t2 = t1;
    if (tpp.v >= (N(2.0) * stepmax - step0).v) {
      stepmax = stepmax * N(2.0);
      if (order != 2) order /= 2;
    }
  }
  return true;
}

// ------------------------------------------------------------------ device side
// Fills a node buffer's float fields from its doubles (the forward kernels read both).
__global__ void k_adj_derive(NodeBufView nb, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  NodeVal v;
  v.x = nb.x[i]; v.y = nb.y[i]; v.z = nb.z[i];
  v.ipx = nb.ipx[i]; v.ipy = nb.ipy[i]; v.ipz = nb.ipz[i]; v.dtau = nb.dtau[i]; v.amp = nb.amp[i];
  store_node(nb, i, v);
}

constexpr int kAdjNodes = 128, kAdjProbes = 512;

// Per node n, over the probes p with upstream gradients g_p = dL/dT_p and the term
// E_pn = w_n exp(-3 (dx^2/phx + dy^2/phy + dz^2/phz)), dx = x_p - x_n:
//   G[0] = sum g E / w                  (dL/dw)
//   G[1..3] = 6 w (1/phx, 1/phy, 1/phz) sum g E/w (dx, dy, dz)     (dL/d node x, y, z)
//   G[4..6] = -3 w sum g E/w (dx^2, dy^2, dz^2)                     (dL/d(1/phx), ...)
// One thread per node and a chunk of probes; each term is recomputed, nothing is stored
// per pair.  FP32 form: the forward's split-float offsets and exp2, Kahan sums per thread;
// chunks meet in FP64 atomics.
template <int PREC>
__global__ void __launch_bounds__(kAdjNodes) k_adjoint(DevProblem P, NodeBufView nb, int n, const int64_t* pts,
                                                       int npts, const double* g, double* G) {
  __shared__ double sP[kAdjProbes][4];
  const int node = blockIdx.x * kAdjNodes + threadIdx.x;
  const int p0 = blockIdx.y * kAdjProbes, np = min(kAdjProbes, npts - p0);
  for (int i = threadIdx.x; i < np; i += kAdjNodes) {
    double x, y, z;
    point_xyz(P, pts[p0 + i], x, y, z);
    sP[i][0] = x; sP[i][1] = y; sP[i][2] = z; sP[i][3] = g[p0 + i];
  }
  __syncthreads();
  if (node >= n) return;
  if (PREC == 0) {
    const double nx = nb.x[node], ny = nb.y[node], nz = nb.z[node];
    const double ipx = nb.ipx[node], ipy = nb.ipy[node], ipz = nb.ipz[node];
    double S[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int i = 0; i < np; ++i) {
      const double dx = sP[i][0] - nx, dy = sP[i][1] - ny, dz = sP[i][2] - nz;
      const double ge = sP[i][3] * exp(-3.0 * (dx * dx * ipx + dy * dy * ipy + dz * dz * ipz));
      S[0] += ge; S[1] += ge * dx; S[2] += ge * dy; S[3] += ge * dz;
      S[4] += ge * dx * dx; S[5] += ge * dy * dy; S[6] += ge * dz * dz;
    }
    const double w = nb.dtau[node] * nb.amp[node];
    atomicAdd(G + 0 * n + node, S[0]);
    atomicAdd(G + 1 * n + node, 6.0 * w * ipx * S[1]);
    atomicAdd(G + 2 * n + node, 6.0 * w * ipy * S[2]);
    atomicAdd(G + 3 * n + node, 6.0 * w * ipz * S[3]);
    atomicAdd(G + 4 * n + node, -3.0 * w * S[4]);
    atomicAdd(G + 5 * n + node, -3.0 * w * S[5]);
    atomicAdd(G + 6 * n + node, -3.0 * w * S[6]);
  } else {
    const float xh = nb.xh[node], xl = nb.xl[node], yh = nb.yh[node], yl = nb.yl[node];
    const float zh = nb.zh[node], zl = nb.zl[node];
    const float kx = nb.kx[node], ky = nb.ky[node], kz = nb.kz[node];
    float s[7] = {0, 0, 0, 0, 0, 0, 0}, c[7] = {0, 0, 0, 0, 0, 0, 0};
    auto kahan = [&](int j, float v) {
      const float y = v - c[j], t = s[j] + y;
      c[j] = (t - s[j]) - y;
      s[j] = t;
    };
    for (int i = 0; i < np; ++i) {
      const float pxh = __double2float_rn(sP[i][0]), pyh = __double2float_rn(sP[i][1]), pzh = __double2float_rn(sP[i][2]);
      const float pxl = __double2float_rn(sP[i][0] - (double)pxh), pyl = __double2float_rn(sP[i][1] - (double)pyh),
                  pzl = __double2float_rn(sP[i][2] - (double)pzh);
      const float dx = (pxh - xh) + (pxl - xl), dy = (pyh - yh) + (pyl - yl), dz = (pzh - zh) + (pzl - zl);
      const float e = fmaf(dz * dz, kz, fmaf(dy * dy, ky, dx * dx * kx));
      const float ge = (float)sP[i][3] * ex2_approx(e);
      kahan(0, ge); kahan(1, ge * dx); kahan(2, ge * dy); kahan(3, ge * dz);
      kahan(4, ge * dx * dx); kahan(5, ge * dy * dy); kahan(6, ge * dz * dz);
    }
    const double w = nb.dtau[node] * nb.amp[node];
    double S[7];
    for (int j = 0; j < 7; ++j) S[j] = (double)s[j] - (double)c[j];
    atomicAdd(G + 0 * n + node, S[0]);
    atomicAdd(G + 1 * n + node, 6.0 * w * nb.ipx[node] * S[1]);
    atomicAdd(G + 2 * n + node, 6.0 * w * nb.ipy[node] * S[2]);
    atomicAdd(G + 3 * n + node, 6.0 * w * nb.ipz[node] * S[3]);
    atomicAdd(G + 4 * n + node, -3.0 * w * S[4]);
    atomicAdd(G + 5 * n + node, -3.0 * w * S[5]);
    atomicAdd(G + 6 * n + node, -3.0 * w * S[6]);
  }
}

}  // namespace

// ------------------------------------------------------------------ the handle
struct th_adj {
  HostProblem hp;
  DevProblem dp{};
  int precision = TH_FP32_KAHAN;
  std::vector<int64_t> probes;
  std::vector<double> times;
  std::vector<double> theta;        // parameters of the last forward
  int nvert = 0;                    // path segments after the origin (vertices)
  std::string err;
  std::vector<TapeEntry> tape;      // the recorded walk of the last backward
  // device (allocated at the first forward)
  int device = -1;
  cudaStream_t stream = nullptr;
  void* node_mem = nullptr;
  NodeBufView nb{};
  int node_cap = 0;
  int64_t* d_probes = nullptr;
  double* d_T = nullptr;
  double* d_g = nullptr;
  double* d_G = nullptr;
  int* d_count = nullptr;
  unsigned long long* d_pairs = nullptr;
};

namespace {

std::string g_adj_error;

th_status afail(th_adj* a, th_status st, const std::string& m) {
  if (a) a->err = m; else g_adj_error = m;
  return st;
}

#define ACUDA(a, call)                                                                       \
  do {                                                                                       \
    const cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) return afail((a), TH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// The walk's inputs for parameters theta; var(x, i) makes parameter i.
template <class N, class Var>
void build_problem(const th_adj& A, const double* th, Var var, DBeam<N>& B, std::vector<DSeg<N>>& path) {
  const N P = var(th[0], 0), eta = var(th[1], 1), ax = var(th[2], 2), ay = var(th[3], 3), az = var(th[4], 4),
          a = var(th[5], 5);
  const N q = (P * eta) * N(2.0);                                // src/Init.cpp:862-865
  B.az = az;
  B.ax2 = ax * ax; B.ay2 = ay * ay; B.az2 = az * az;
  B.nond = (ax * ax) / a;
  B.beta = (N(std::pow(3.0 / 3.14159265358979323846, 1.5)) * q) / N(A.hp.rho * A.hp.cps);
  B.a12 = N(12.0) * a;
  const std::vector<DevSeg>& hpath = A.hp.paths[0];
  path.assign(hpath.size(), DSeg<N>());
  for (size_t k = 0; k < hpath.size(); ++k) {
    DSeg<N>& s = path[k];
    s.mode = hpath[k].mode; s.q = hpath[k].q; s.prm = hpath[k].prm;
    if (k == 0) { s.x = N(hpath[0].x); s.y = N(hpath[0].y); s.z = N(hpath[0].z); s.tend = N(0.0); continue; }
    s.x = var(th[6 + 2 * (k - 1)], 6 + 2 * (int)(k - 1));
    s.y = var(th[7 + 2 * (k - 1)], 7 + 2 * (int)(k - 1));
    s.z = N(hpath[k].z);
    if (s.mode) s.tend = path[k - 1].tend + N(s.prm);         // src/Init.cpp path times
    else {
      const N dx = s.x - path[k - 1].x, dy = s.y - path[k - 1].y, dz = s.z - path[k - 1].z;
      s.tend = path[k - 1].tend + dsqrt((dx * dx + dy * dy) + dz * dz) / N(s.prm);
    }
    s.rt0 = s.mode == 0 ? (N(0.58870501125) * ax) / N(s.prm) : N(0.0);
  }
  B.tlast = path.back().tend;
  B.nseg = (int)path.size();
}

template <class N, class Var>
th_status node_lists(th_adj* A, const double* th, Var var, std::vector<std::vector<DNode<N>>>& lists) {
  DBeam<N> B;
  std::vector<DSeg<N>> path;
  build_problem<N>(*A, th, var, B, path);
  lists.assign(A->times.size(), {});
  for (size_t i = 0; i < A->times.size(); ++i)
    if (!walk_nodes(A->dp, B, path, A->times[i], false, lists[i]))
      return afail(A, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
  return TH_OK;
}

th_status ensure_device(th_adj* A, int nmax) {
  if (A->device < 0) {
    ACUDA(A, cudaGetDevice(&A->device));
    ACUDA(A, cudaStreamCreateWithFlags(&A->stream, cudaStreamNonBlocking));
    const size_t np = A->probes.size();
    ACUDA(A, cudaMalloc(&A->d_probes, np * sizeof(int64_t)));
    ACUDA(A, cudaMemcpy(A->d_probes, A->probes.data(), np * sizeof(int64_t), cudaMemcpyHostToDevice));
    ACUDA(A, cudaMalloc(&A->d_T, std::max<size_t>(np, 1) * sizeof(double)));
    ACUDA(A, cudaMalloc(&A->d_g, std::max<size_t>(np, 1) * sizeof(double)));
    ACUDA(A, cudaMalloc(&A->d_count, sizeof(int)));
    ACUDA(A, cudaMalloc(&A->d_pairs, sizeof(unsigned long long)));
    ACUDA(A, cudaMemset(A->d_pairs, 0, sizeof(unsigned long long)));
  }
  ACUDA(A, cudaSetDevice(A->device));
  if (nmax > A->node_cap) {
    const int cap = ((nmax + 255) / 256) * 256;
    cudaFree(A->node_mem);
    cudaFree(A->d_G);
    A->node_mem = nullptr;
    A->d_G = nullptr;
    ACUDA(A, cudaMalloc(&A->node_mem, (size_t)cap * (8 * sizeof(double) + 10 * sizeof(float))));
    ACUDA(A, cudaMalloc(&A->d_G, (size_t)7 * cap * sizeof(double)));
    double* d = (double*)A->node_mem;
    float* f = (float*)(d + 8 * (size_t)cap);
    NodeBufView& nb = A->nb;
    nb.cap = cap;
    nb.x = d; nb.y = d + cap; nb.z = d + 2 * (size_t)cap; nb.ipx = d + 3 * (size_t)cap; nb.ipy = d + 4 * (size_t)cap;
    nb.ipz = d + 5 * (size_t)cap; nb.dtau = d + 6 * (size_t)cap; nb.amp = d + 7 * (size_t)cap;
    nb.kx = f; nb.ky = f + cap; nb.kz = f + 2 * (size_t)cap; nb.w = f + 3 * (size_t)cap; nb.xh = f + 4 * (size_t)cap;
    nb.xl = f + 5 * (size_t)cap; nb.yh = f + 6 * (size_t)cap; nb.yl = f + 7 * (size_t)cap; nb.zh = f + 8 * (size_t)cap;
    nb.zl = f + 9 * (size_t)cap;
    A->node_cap = cap;
  }
  return TH_OK;
}

// Uploads one node list's values and derives the float fields (enqueued on the stream).
template <class N>
th_status upload_nodes(th_adj* A, const std::vector<DNode<N>>& L) {
  const int n = (int)L.size();
  std::vector<double> h((size_t)8 * n);
  for (int i = 0; i < n; ++i) {
    const DNode<N>& v = L[i];
    const double f[8] = {v.x.v, v.y.v, v.z.v, v.ipx.v, v.ipy.v, v.ipz.v, v.dtau.v, v.amp.v};
    for (int j = 0; j < 8; ++j) h[(size_t)j * n + i] = f[j];
  }
  double* dst[8] = {A->nb.x, A->nb.y, A->nb.z, A->nb.ipx, A->nb.ipy, A->nb.ipz, A->nb.dtau, A->nb.amp};
  for (int j = 0; j < 8; ++j)
    ACUDA(A, cudaMemcpyAsync(dst[j], h.data() + (size_t)j * n, n * sizeof(double), cudaMemcpyHostToDevice, A->stream));
  if (n > 0) k_adj_derive<<<(n + 255) / 256, 256, 0, A->stream>>>(A->nb, n);
  ACUDA(A, cudaMemcpyAsync(A->d_count, &n, sizeof(int), cudaMemcpyHostToDevice, A->stream));
  ACUDA(A, cudaStreamSynchronize(A->stream));      // h and n leave scope
  return TH_OK;
}

auto constant_var = [](double x, int) { return Rev(x); };

}  // namespace

extern "C" {

th_status th_adj_create(const char* param_input, int32_t precision, const int64_t* probes, int32_t nprobe,
                        const double* times, int32_t ntimes, th_adj** out) {
  if (!param_input || !probes || nprobe <= 0 || !times || ntimes <= 0 || !out)
    return afail(nullptr, TH_ERR_INVALID, "bad argument");
  if (precision != TH_FP64 && precision != TH_FP32_KAHAN) return afail(nullptr, TH_ERR_INVALID, "unknown precision");
  *out = nullptr;
  th_adj* A = new th_adj();
  std::string e;
  if (!th_load_deck(param_input, A->hp, e)) { delete A; return afail(nullptr, TH_ERR_INVALID, e); }
  if (A->hp.beams.size() != 1) { delete A; return afail(nullptr, TH_ERR_UNSUPPORTED, "the adjoint takes single-beam decks"); }
  if (A->hp.custom) { delete A; return afail(nullptr, TH_ERR_UNSUPPORTED, "the adjoint takes grid decks (probes are grid points)"); }
  if (A->hp.compress) {
    delete A;
    return afail(nullptr, TH_ERR_UNSUPPORTED, "the adjoint takes decks without path compression");
  }
  A->precision = precision;
  th_make_dev_problem(A->hp, nullptr, A->dp);
  if (A->dp.n_images > 1) { delete A; return afail(nullptr, TH_ERR_UNSUPPORTED, "the adjoint takes decks without reflections"); }
  for (int i = 0; i < nprobe; ++i)
    if (probes[i] < 0 || probes[i] >= A->hp.pnum) { delete A; return afail(nullptr, TH_ERR_INVALID, "probe point out of the grid"); }
  for (int i = 0; i < ntimes; ++i)
    if (!(times[i] >= 0.0)) { delete A; return afail(nullptr, TH_ERR_INVALID, "times must be >= 0"); }
  A->probes.assign(probes, probes + nprobe);
  A->times.assign(times, times + ntimes);
  A->nvert = (int)A->hp.paths[0].size() - 1;
  A->theta.resize(6 + 2 * A->nvert);
  th_adj_params(A, A->theta.data());
  *out = A;
  return TH_OK;
}

void th_adj_destroy(th_adj* A) {
  if (!A) return;
  if (A->device >= 0) cudaSetDevice(A->device);
  if (A->stream) cudaStreamSynchronize(A->stream);
  cudaFree(A->node_mem); cudaFree(A->d_probes); cudaFree(A->d_T); cudaFree(A->d_g); cudaFree(A->d_G);
  cudaFree(A->d_count); cudaFree(A->d_pairs);
  if (A->stream) cudaStreamDestroy(A->stream);
  delete A;
}

const char* th_adj_last_error(const th_adj* A) { return A ? A->err.c_str() : g_adj_error.c_str(); }

int32_t th_adj_num_params(const th_adj* A) { return A ? 6 + 2 * A->nvert : 0; }

th_status th_adj_params(th_adj* A, double* theta) {
  if (!A || !theta) return afail(A, TH_ERR_INVALID, "null argument");
  const HostBeam& B = A->hp.beams[0];
  theta[0] = B.power; theta[1] = B.eff; theta[2] = B.ax; theta[3] = B.ay; theta[4] = B.az; theta[5] = A->hp.a;
  for (int k = 1; k <= A->nvert; ++k) {
    theta[6 + 2 * (k - 1)] = A->hp.paths[0][k].x;
    theta[7 + 2 * (k - 1)] = A->hp.paths[0][k].y;
  }
  return TH_OK;
}

th_status th_adj_host_nodes(th_adj* A, const double* theta, int32_t time_idx, double* out, int32_t cap,
                            double* tangents, int32_t* n_out) {
  if (!A || !theta || !n_out || time_idx < 0 || time_idx >= (int)A->times.size())
    return afail(A, TH_ERR_INVALID, "bad argument");
  const int np = tangents ? th_adj_num_params(A) : 0;
  auto var = [np](double x, int i) {
    Dual r(x);
    if (np) { r.d.assign(np, 0.0); r.d[i] = 1.0; }
    return r;
  };
  std::vector<std::vector<DNode<Dual>>> lists;
  const std::vector<double> keep = A->times;
  A->times.assign(1, keep[time_idx]);
  th_status st = node_lists<Dual>(A, theta, var, lists);
  A->times = keep;
  if (st != TH_OK) return st;
  const std::vector<DNode<Dual>>& L = lists[0];
  *n_out = (int)L.size();
  const int n = std::min<int>((int)L.size(), cap);
  for (int i = 0; i < n; ++i) {
    const Dual* f[8] = {&L[i].x, &L[i].y, &L[i].z, &L[i].ipx, &L[i].ipy, &L[i].ipz, &L[i].dtau, &L[i].amp};
    for (int j = 0; j < 8; ++j) {
      if (out) out[(size_t)j * cap + i] = f[j]->v;
      if (tangents)
        for (int k = 0; k < np; ++k)
          tangents[((size_t)j * cap + i) * np + k] = f[j]->d.empty() ? 0.0 : f[j]->d[k];
    }
  }
  return TH_OK;
}

th_status th_adj_forward(th_adj* A, const double* theta, double* T_out) {
  if (!A || !theta || !T_out) return afail(A, TH_ERR_INVALID, "null argument");
  std::vector<std::vector<DNode<Rev>>> lists;
  th_status st = node_lists<Rev>(A, theta, constant_var, lists);   // values only: nothing recorded
  if (st != TH_OK) return st;
  A->theta.assign(theta, theta + th_adj_num_params(A));
  int nmax = 1;
  for (const auto& L : lists) nmax = std::max<int>(nmax, (int)L.size());
  if ((st = ensure_device(A, nmax)) != TH_OK) return st;
  const int64_t np = (int64_t)A->probes.size();
  for (size_t i = 0; i < lists.size(); ++i) {
    if ((st = upload_nodes(A, lists[i])) != TH_OK) return st;
    th_launch_list_sum(A->dp, A->nb, A->d_count, A->d_probes, np, A->d_T, A->precision, A->d_pairs, A->stream);
    ACUDA(A, cudaGetLastError());
    ACUDA(A, cudaMemcpyAsync(T_out + i * np, A->d_T, np * sizeof(double), cudaMemcpyDeviceToHost, A->stream));
    ACUDA(A, cudaStreamSynchronize(A->stream));
  }
  return TH_OK;
}

th_status th_adj_backward(th_adj* A, const double* dL_dT, double* dL_dtheta) {
  if (!A || !dL_dT || !dL_dtheta) return afail(A, TH_ERR_INVALID, "null argument");
  const int npar = th_adj_num_params(A);
  // re-walk at the last forward's theta, recording every operation; the parameters are the
  // tape's first npar entries
  A->tape.clear();
  A->tape.reserve(1 << 20);
  for (int j = 0; j < npar; ++j) A->tape.push_back({-1, -1, 0.0, 0.0});
  g_tape = &A->tape;
  auto var = [](double x, int i) { Rev r(x); r.i = i; return r; };
  std::vector<std::vector<DNode<Rev>>> lists;
  th_status st = node_lists<Rev>(A, A->theta.data(), var, lists);
  g_tape = nullptr;
  if (st != TH_OK) return st;
  int nmax = 1;
  for (const auto& L : lists) nmax = std::max<int>(nmax, (int)L.size());
  if ((st = ensure_device(A, nmax)) != TH_OK) return st;
  std::vector<double> adj(A->tape.size(), 0.0);
  auto seed = [&](const Rev& q, double g) { if (q.i >= 0) adj[q.i] += g; };
  const int np = (int)A->probes.size();
  std::vector<double> G;
  for (size_t i = 0; i < lists.size(); ++i) {
    const std::vector<DNode<Rev>>& L = lists[i];
    const int n = (int)L.size();
    if (n == 0) continue;
    if ((st = upload_nodes(A, L)) != TH_OK) return st;
    ACUDA(A, cudaMemcpyAsync(A->d_g, dL_dT + i * np, np * sizeof(double), cudaMemcpyHostToDevice, A->stream));
    ACUDA(A, cudaMemsetAsync(A->d_G, 0, (size_t)7 * n * sizeof(double), A->stream));
    const dim3 grid((n + kAdjNodes - 1) / kAdjNodes, (np + kAdjProbes - 1) / kAdjProbes);
    if (A->precision == TH_FP64)
      k_adjoint<0><<<grid, kAdjNodes, 0, A->stream>>>(A->dp, A->nb, n, A->d_probes, np, A->d_g, A->d_G);
    else
      k_adjoint<1><<<grid, kAdjNodes, 0, A->stream>>>(A->dp, A->nb, n, A->d_probes, np, A->d_g, A->d_G);
    ACUDA(A, cudaGetLastError());
    G.resize((size_t)7 * n);
    ACUDA(A, cudaMemcpyAsync(G.data(), A->d_G, (size_t)7 * n * sizeof(double), cudaMemcpyDeviceToHost, A->stream));
    ACUDA(A, cudaStreamSynchronize(A->stream));
    // the loss gradient with respect to each node quantity (w = dtau * amp)
    for (int k = 0; k < n; ++k) {
      const DNode<Rev>& v = L[k];
      const double gw = G[(size_t)0 * n + k];
      seed(v.dtau, gw * v.amp.v);
      seed(v.amp, gw * v.dtau.v);
      seed(v.x, G[(size_t)1 * n + k]);
      seed(v.y, G[(size_t)2 * n + k]);
      seed(v.z, G[(size_t)3 * n + k]);
      seed(v.ipx, G[(size_t)4 * n + k]);
      seed(v.ipy, G[(size_t)5 * n + k]);
      seed(v.ipz, G[(size_t)6 * n + k]);
    }
  }
  // reverse sweep over the recorded walk
  for (size_t i = A->tape.size(); i-- > (size_t)npar;) {
    const double g = adj[i];
    if (g == 0.0) continue;
    const TapeEntry& e = A->tape[i];
    if (e.a >= 0) adj[e.a] += e.da * g;
    if (e.b >= 0) adj[e.b] += e.db * g;
  }
  for (int j = 0; j < npar; ++j) dL_dtheta[j] = adj[j];
  return TH_OK;
}

}  // extern "C"
