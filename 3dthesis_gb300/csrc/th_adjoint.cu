// Adjoint of probe temperatures for calibration: dL/d{P, eta, Width_X, Width_Y, Depth_Z,
// alpha} and dL/d(path vertex x, y) of a single-beam problem, for a loss L of the
// temperatures at probe points and times.
//
// The node list is a function of the parameters through the quadrature walk: node times,
// weights and positions move with the widths, the diffusivity and the segment end times
// (which follow the vertices through the segment lengths).  The host re-walks the path in
// forward-mode dual numbers - the same FP64 operations in the same order as the device walk
// (src/Calc.cpp:67-211, src/Util.cpp:192-237), so the values are the device's node list
// bit for bit - and carries each node quantity's derivative with respect to every
// parameter.  The device kernel recomputes every probe x node term (no pair storage) and
// sums, per node, the loss gradient with respect to the node's position, inverse widths and
// weight; the host contracts those with the node tangents.  Discrete choices of the walk
// (interval counts, Gauss orders, the r_max cut-off) are held fixed, as a finite difference
// that does not cross one of them sees.
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

// ------------------------------------------------------------------ dual numbers
// Value and gradient over the parameter vector; an empty gradient is a constant.
struct Dual {
  double v = 0.0;
  std::vector<double> d;
  Dual() = default;
  Dual(double x) : v(x) {}
};

Dual variable(double x, int i, int np) {
  Dual r(x);
  r.d.assign(np, 0.0);
  r.d[i] = 1.0;
  return r;
}

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

// ------------------------------------------------------------------ the walk in duals
struct DSeg { Dual x, y, z, tend, rt0; double q, prm; int mode; };
struct DBeam { Dual az, ax2, ay2, az2, nond, beta, tlast, a12; int nseg; };

struct DNode { Dual x, y, z, ipx, ipy, ipz, dtau, amp; };

struct DWalk {
  double t;
  Dual t1, t2, tpp, stepmax, step0;
  int s, order;
  bool more, sw;
};

// src/Util.cpp:192-209
Dual ref_time(const DBeam& B, const std::vector<DSeg>& path, const Dual& tpp, int s) {
  Dual spp = tpp / B.nond;
  if (spp.v < 0.0) spp = Dual(0.0);
  if (path[s].mode == 0) return path[s].rt0 * dsqrt(Dual(12.0) * spp + Dual(1.0));
  Dual r = path[s].tend - path[s - 1].tend;
  if (r.v == 0) r = Dual(1.0e-9);
  return r;
}

int find_seg(const std::vector<DSeg>& path, double t) {
  int lo = 1, hi = (int)path.size() - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (t > path[mid].tend.v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

struct DLoc { Dual x, y, z; double q; };

// src/Util.cpp:211-237 with the r_max cut-off of src/Util.cpp:168-172
DLoc beam_loc(const DevProblem& P, const std::vector<DSeg>& path, const Dual& t, int s) {
  const DSeg& cur = path[s];
  DLoc L;
  if (cur.mode) {
    L.x = cur.x; L.y = cur.y; L.z = cur.z;
  } else {
    const DSeg& prv = path[s - 1];
    const Dual r = (t - prv.tend) / (cur.tend - prv.tend);
    L.x = prv.x + r * (cur.x - prv.x);
    L.y = prv.y + r * (cur.y - prv.y);
    L.z = prv.z + r * (cur.z - prv.z);
  }
  const bool out = (L.x.v > P.rx1) || (L.x.v < P.rx0) || (L.y.v > P.ry1) || (L.y.v < P.ry0);
  L.q = out ? 0.0 : cur.q;
  return L;
}

DNode finish_node(const DBeam& B, const Dual& ct, const Dual& qb, const Dual& dtau, const DLoc& L) {
  const Dual phx = B.ax2 + ct, phy = B.ay2 + ct, phz = B.az2 + ct;
  DNode v;
  v.x = L.x; v.y = L.y; v.z = L.z;
  v.ipx = Dual(1.0) / phx; v.ipy = Dual(1.0) / phy; v.ipz = Dual(1.0) / phz;
  v.dtau = dtau;
  v.amp = qb / dsqrt((phx * phy) * phz);
  return v;
}

// The node list at t in the device's order (zero-weight node, then each interval's Gauss
// points from the late end); returns false when the walk exceeds its step limit.
bool walk_nodes(const DevProblem& P, const DBeam& B, const std::vector<DSeg>& path, double t, bool is_sol,
                std::vector<DNode>& out) {
  DWalk W;
  W.t = t;
  W.s = find_seg(path, t);
  W.step0 = is_sol ? B.nond * B.az : B.nond;
  W.stepmax = W.step0;
  W.order = 16;
  W.t2 = Dual(t); W.t1 = Dual(t); W.tpp = Dual(0.0);
  if (t > B.tlast.v) { W.tpp = W.tpp + (Dual(t) - B.tlast); W.t2 = B.tlast; }
  int guard = 0;
  while (W.tpp.v >= (Dual(2.0) * W.stepmax - W.step0).v && guard++ < 4096) {
    W.stepmax = W.stepmax * Dual(2.0);
    if (W.order != 2) W.order /= 2;
  }
  W.more = true;
  W.sw = false;
  {  // src/Calc.cpp:124-132
    const DLoc L = beam_loc(P, path, Dual(t), W.s);
    if (t <= B.tlast.v && L.q * B.beta.v > 0.0) out.push_back(finish_node(B, Dual(0.0), Dual(L.q) * B.beta, Dual(0.0), L));
  }
  int steps = 0;
  while (W.more) {
    if (++steps > kMaxWalkSteps) return false;
    const Dual rt = ref_time(B, path, W.tpp, W.s);
    const Dual use = (rt.v < W.stepmax.v) ? rt : W.stepmax;
    W.t1 = W.t2 - use;
    const Dual next = path[W.s - 1].tend;
    W.sw = false;
    if (W.t1.v <= next.v) {
      W.t1 = next;
      if (next.v > 0.0) W.sw = true; else W.more = false;
    }
    const int base = W.order - 2;
    for (int k = base + W.order - 1; k >= base; --k) {       // src/Calc.cpp:176-190
      const Dual h = W.t2 - W.t1;
      const Dual tp = Dual(0.5) * ((h * Dual(P.gl_loc[k])) + (W.t2 + W.t1));
      const Dual ct = B.a12 * (Dual(t) - tp);
      const DLoc L = beam_loc(P, path, tp, W.s);
      const Dual qb = Dual(L.q) * B.beta;
      const Dual dtau = (Dual(0.5) * h) * Dual(P.gl_w[k]);
      if (!(qb.v > 0.0 && dtau.v > 0.0)) continue;
      out.push_back(finish_node(B, ct, qb, dtau, L));
    }
    if (W.sw) W.s--;                                           // src/Calc.cpp:192-207
    W.tpp = W.tpp + (W.t2 - W.t1);
    W.t2 = W.t1;
    if (W.tpp.v >= (Dual(2.0) * W.stepmax - W.step0).v) {
      W.stepmax = W.stepmax * Dual(2.0);
      if (W.order != 2) W.order /= 2;
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

// The dual problem for parameters theta (gradients only when np > 0).
void build_dual(const th_adj& A, const double* th, int np, DBeam& B, std::vector<DSeg>& path) {
  auto var = [&](double x, int i) { return np ? variable(x, i, np) : Dual(x); };
  const Dual P = var(th[0], 0), eta = var(th[1], 1), ax = var(th[2], 2), ay = var(th[3], 3), az = var(th[4], 4),
             a = var(th[5], 5);
  const Dual q = (P * eta) * Dual(2.0);                           // src/Init.cpp:862-865
  B.az = az;
  B.ax2 = ax * ax; B.ay2 = ay * ay; B.az2 = az * az;
  B.nond = (ax * ax) / a;
  B.beta = (Dual(std::pow(3.0 / 3.14159265358979323846, 1.5)) * q) / Dual(A.hp.rho * A.hp.cps);
  B.a12 = Dual(12.0) * a;
  const std::vector<DevSeg>& hpath = A.hp.paths[0];
  path.assign(hpath.size(), DSeg());
  for (size_t k = 0; k < hpath.size(); ++k) {
    DSeg& s = path[k];
    s.mode = hpath[k].mode; s.q = hpath[k].q; s.prm = hpath[k].prm;
    if (k == 0) { s.x = Dual(hpath[0].x); s.y = Dual(hpath[0].y); s.z = Dual(hpath[0].z); s.tend = Dual(0.0); continue; }
    s.x = var(th[6 + 2 * (k - 1)], 6 + 2 * (int)(k - 1));
    s.y = var(th[7 + 2 * (k - 1)], 7 + 2 * (int)(k - 1));
    s.z = Dual(hpath[k].z);
    if (s.mode) s.tend = path[k - 1].tend + Dual(s.prm);
    else {
      const Dual dx = s.x - path[k - 1].x, dy = s.y - path[k - 1].y, dz = s.z - path[k - 1].z;
      s.tend = path[k - 1].tend + dsqrt((dx * dx + dy * dy) + dz * dz) / Dual(s.prm);
    }
    s.rt0 = s.mode == 0 ? (Dual(0.58870501125) * ax) / Dual(s.prm) : Dual(0.0);
  }
  B.tlast = path.back().tend;
  B.nseg = (int)path.size();
}

th_status node_lists(th_adj* A, const double* th, int np, std::vector<std::vector<DNode>>& lists) {
  DBeam B;
  std::vector<DSeg> path;
  build_dual(*A, th, np, B, path);
  // the walk's DevProblem fields that do not follow the parameters: Gauss tables, r_max box,
  // Depth_Z of the solidification schedule
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
th_status upload_nodes(th_adj* A, const std::vector<DNode>& L) {
  const int n = (int)L.size();
  std::vector<double> h((size_t)8 * n);
  for (int i = 0; i < n; ++i) {
    const DNode& v = L[i];
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
  std::vector<std::vector<DNode>> lists;
  const std::vector<double> keep = A->times;
  A->times.assign(1, keep[time_idx]);
  th_status st = node_lists(A, theta, np, lists);
  A->times = keep;
  if (st != TH_OK) return st;
  const std::vector<DNode>& L = lists[0];
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
  std::vector<std::vector<DNode>> lists;
  th_status st = node_lists(A, theta, 0, lists);
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
  std::vector<std::vector<DNode>> lists;
  th_status st = node_lists(A, A->theta.data(), npar, lists);   // recomputed with tangents
  if (st != TH_OK) return st;
  int nmax = 1;
  for (const auto& L : lists) nmax = std::max<int>(nmax, (int)L.size());
  if ((st = ensure_device(A, nmax)) != TH_OK) return st;
  std::fill(dL_dtheta, dL_dtheta + npar, 0.0);
  const int np = (int)A->probes.size();
  std::vector<double> G;
  for (size_t i = 0; i < lists.size(); ++i) {
    const std::vector<DNode>& L = lists[i];
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
    // chain: dL/dtheta += sum_n G . d(node)/dtheta, with w = dtau * amp
    for (int k = 0; k < n; ++k) {
      const DNode& v = L[k];
      const double gw = G[(size_t)0 * n + k];
      auto add = [&](double coef, const Dual& q) {
        if (coef == 0.0 || q.d.empty()) return;
        for (int j = 0; j < npar; ++j) dL_dtheta[j] += coef * q.d[j];
      };
      add(gw * v.amp.v, v.dtau);
      add(gw * v.dtau.v, v.amp);
      add(G[(size_t)1 * n + k], v.x);
      add(G[(size_t)2 * n + k], v.y);
      add(G[(size_t)3 * n + k], v.z);
      add(G[(size_t)4 * n + k], v.ipx);
      add(G[(size_t)5 * n + k], v.ipy);
      add(G[(size_t)6 * n + k], v.ipz);
    }
  }
  return TH_OK;
}

}  // extern "C"
