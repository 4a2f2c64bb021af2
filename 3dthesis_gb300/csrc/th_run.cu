// Mode drivers behind th_simulate / th_solidify / th_field.
//
// Solidification (src/Run.cpp:390-709) runs in windows of steps: the host lays out the
// step times exactly as the reference accumulates them (t += dt), one kernel builds the
// window's node lists (one warp per step), then either the persistent tracking kernel
// (Volume / Surface) or one whole-grid kernel per step (NoTracking) advances the state,
// and the queued liquid -> solid records are solidified in bulk.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "th_ctx.h"
#include "th_output.h"
#include "th_track.h"

namespace {

enum { F_T, F_TSOL, F_G, F_V, F_GX, F_GY, F_GZ, F_DTDT, F_EQ, F_NUMMELT, F_DEPTH, F_FLAG };

constexpr int kWindowTrack = 256;     // steps per node window (tracking)
constexpr int kWindowNoTrack = 32;    // steps per node window (NoTracking: whole grid per step)
constexpr int kRecCap = 1 << 22;      // queued solidification records

}  // namespace

struct RunState {
  TrackState S{};
  std::vector<void*> allocs;
  std::vector<std::pair<size_t, int>> alloc_fill;   // bytes and fill byte of each allocation
  void* win_mem = nullptr;
  NodeWindow W{};
  double* d_t = nullptr;
  int* d_count = nullptr;
  int win_slots = 0;
  int slot_cap = 1024;
  int k = 0;              // next step
  double t_prev = 0.0;    // time of step k - 1
  double t_next = 0.0;    // time of step k
  bool done = false;
  bool initialised = false;
  int max_rounds = 0;
  double* d_field = nullptr;
  // device time per phase (ms) and counts, for th_run_stats
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaEvent_t ev_run[2] = {nullptr, nullptr};
  double ms_nodes = 0, ms_track = 0, ms_solid = 0, ms_device = 0;
  long long windows = 0, records = 0;
};

void th_release_run_state(th_ctx* ctx) {
  RunState* r = ctx->run;
  if (!r) return;
  for (void* p : r->allocs) cudaFree(p);
  cudaFree(r->win_mem);
  cudaFree(r->d_t);
  cudaFree(r->d_count);
  cudaFree(r->d_field);
  if (r->ev[0]) cudaEventDestroy(r->ev[0]);
  if (r->ev[1]) cudaEventDestroy(r->ev[1]);
  if (r->ev_run[0]) cudaEventDestroy(r->ev_run[0]);
  if (r->ev_run[1]) cudaEventDestroy(r->ev_run[1]);
  delete r;
  ctx->run = nullptr;
}

namespace {

template <class T>
th_status dalloc(th_ctx* ctx, RunState* r, T** p, size_t n, int fill_byte = 0) {
  void* v = nullptr;
  th_status st = th_cuda_check(ctx, cudaMalloc(&v, std::max<size_t>(n, 1) * sizeof(T)), "cudaMalloc");
  if (st != TH_OK) return st;
  r->allocs.push_back(v);
  r->alloc_fill.push_back({std::max<size_t>(n, 1) * sizeof(T), fill_byte});
  st = th_cuda_check(ctx, cudaMemsetAsync(v, fill_byte, std::max<size_t>(n, 1) * sizeof(T), ctx->stream), "cudaMemset");
  *p = (T*)v;
  return st;
}

__global__ void k_fill_d(double* a, int64_t n, double v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] = v;
}

th_status init_run(th_ctx* ctx) {
  const HostProblem& hp = ctx->hp;
  if (hp.pnum >= INT_MAX) return th_fail(ctx, TH_ERR_CAPACITY, "solidification needs fewer than 2^31 points");
  RunState* r = new RunState();
  ctx->run = r;
  TrackState& S = r->S;
  const size_t n = (size_t)hp.pnum;
  const size_t ncol = (size_t)hp.nx * hp.ny;
  th_status st = TH_OK;
#define ALLOC(ptr, cnt, fill) if ((st = dalloc(ctx, r, &(ptr), (cnt), (fill))) != TH_OK) return st
  ALLOC(S.T, n, 0);
  ALLOC(S.T_last, n, 0);
  ALLOC(S.stamp, n, 0);
  ALLOC(S.outflag, n, 0);
  ALLOC(S.last_liq, n, 0xff);   // -1
  ALLOC(S.num_melt, n, 0);
  ALLOC(S.sol_step, n, 0xff);   // -1
  if (hp.o_tSol) ALLOC(S.tSol, n, 0);
  if (hp.o_G) ALLOC(S.G, n, 0);
  if (hp.o_V) ALLOC(S.V, n, 0);
  if (hp.o_Gx) ALLOC(S.Gx, n, 0);
  if (hp.o_Gy) ALLOC(S.Gy, n, 0);
  if (hp.o_Gz) ALLOC(S.Gz, n, 0);
  if (hp.o_dTdt) ALLOC(S.dTdt, n, 0);
  if (hp.o_eqFrac) ALLOC(S.eqFrac, n, 0);
  if (hp.tracking == TH_TRACK_SURFACE) {
    if (hp.o_depth) ALLOC(S.depth, n, 0);
    ALLOC(S.depths, ncol, 0);
    ALLOC(S.depth_max, ncol, 0);
  }
  if (hp.tracking != TH_TRACK_NONE) {
    S.list_cap = (int)n;
    for (int i = 0; i < 3; ++i) ALLOC(S.liq[i], n, 0);
    // work items of one step: every claimed point, column layer and depth walk at most
    // once, which in practice stays far below 2 * pnum
    S.queue_cap = (int)std::min<size_t>(2 * n + 4096, (size_t)1 << 24);
    ALLOC(S.queue, (size_t)S.queue_cap, 0);
  }
  S.rec_cap = kRecCap;
  ALLOC(S.rec, (size_t)kRecCap, 0);
  ALLOC(S.C, 1, 0);
  ALLOC(S.bar, 2, 0);
  ALLOC(S.err, 1, 0);
#undef ALLOC
  S.pairs = ctx->d_pairs;
  if (hp.tracking == TH_TRACK_NONE) {                 // NoTracking starts every point at T_0
    k_fill_d<<<1024, 256, 0, ctx->stream>>>(S.T, (int64_t)n, hp.T0);
    st = th_cuda_check(ctx, cudaGetLastError(), "fill");
    if (st != TH_OK) return st;
  }
  r->k = 0;
  r->t_prev = 0.0;
  r->t_next = 0.0;
  r->initialised = true;
  cudaEventCreate(&r->ev[0]);
  cudaEventCreate(&r->ev[1]);
  cudaEventCreate(&r->ev_run[0]);
  cudaEventCreate(&r->ev_run[1]);
  return th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "init");
}

th_status alloc_window(th_ctx* ctx, RunState* r, int slots, int slot_cap) {
  cudaFree(r->win_mem); r->win_mem = nullptr;
  cudaFree(r->d_t); r->d_t = nullptr;
  cudaFree(r->d_count); r->d_count = nullptr;
  const size_t cap = (size_t)slots * slot_cap;
  th_status st = th_cuda_check(ctx, cudaMalloc(&r->win_mem, cap * (8 * sizeof(double) + 10 * sizeof(float))), "cudaMalloc");
  if (st != TH_OK) return st;
  st = th_cuda_check(ctx, cudaMalloc(&r->d_t, slots * sizeof(double)), "cudaMalloc");
  if (st != TH_OK) return st;
  st = th_cuda_check(ctx, cudaMalloc(&r->d_count, slots * sizeof(int)), "cudaMalloc");
  if (st != TH_OK) return st;
  double* d = (double*)r->win_mem;
  float* f = (float*)(d + 8 * cap);
  NodeBufView& nb = r->W.nb;
  nb.cap = (int)cap;
  nb.x = d; nb.y = d + cap; nb.z = d + 2 * cap; nb.ipx = d + 3 * cap; nb.ipy = d + 4 * cap; nb.ipz = d + 5 * cap;
  nb.dtau = d + 6 * cap; nb.amp = d + 7 * cap;
  nb.kx = f; nb.ky = f + cap; nb.kz = f + 2 * cap; nb.w = f + 3 * cap; nb.xh = f + 4 * cap; nb.xl = f + 5 * cap;
  nb.yh = f + 6 * cap; nb.yl = f + 7 * cap; nb.zh = f + 8 * cap; nb.zl = f + 9 * cap;
  r->W.slot_cap = slot_cap;
  r->W.nslots = slots;
  r->W.count = r->d_count;
  r->W.t = r->d_t;
  r->win_slots = slots;
  r->slot_cap = slot_cap;
  return TH_OK;
}

// Builds the node lists of steps [k, k + n) (slots 1..n) and of step k - 1 (slot 0).
th_status build_window(th_ctx* ctx, RunState* r, int n, std::vector<double>& ts) {
  const HostProblem& hp = ctx->hp;
  ts.assign(n + 1, 0.0);
  ts[0] = r->t_prev;
  double t = r->t_next;
  for (int i = 1; i <= n; ++i) { ts[i] = t; t = t + hp.dt; }
  for (int attempt = 0; attempt < 4; ++attempt) {
    if (!r->win_mem || r->win_slots < n + 1) {
      th_status st = alloc_window(ctx, r, std::max(n + 1, r->win_slots), r->slot_cap);
      if (st != TH_OK) return st;
    }
    r->W.base = r->k;
    th_status st = th_cuda_check(ctx, cudaMemcpyAsync(r->d_t, ts.data(), (n + 1) * sizeof(double),
                                                      cudaMemcpyHostToDevice, ctx->stream), "cudaMemcpyAsync");
    if (st != TH_OK) return st;
    st = th_cuda_check(ctx, cudaMemsetAsync(ctx->d_small + 1, 0, sizeof(int), ctx->stream), "cudaMemsetAsync");
    if (st != TH_OK) return st;
    const int first = r->k == 0 ? 1 : 0;
    cudaEventRecord(r->ev[0], ctx->stream);
    th_launch_nodes_window(ctx->dp, r->W, first, n + 1 - first, false, ctx->d_small + 1, ctx->stream);
    cudaEventRecord(r->ev[1], ctx->stream);
    st = th_cuda_check(ctx, cudaGetLastError(), "node window");
    if (st != TH_OK) return st;
    int err = 0;
    std::vector<int> cnt(n + 1);
    st = th_cuda_check(ctx, cudaMemcpyAsync(&err, ctx->d_small + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "copy");
    if (st != TH_OK) return st;
    st = th_cuda_check(ctx, cudaMemcpyAsync(cnt.data(), r->d_count, (n + 1) * sizeof(int), cudaMemcpyDeviceToHost,
                                            ctx->stream), "copy");
    if (st != TH_OK) return st;
    st = th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "node window");
    if (st != TH_OK) return st;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r->ev[0], r->ev[1]);
    r->ms_nodes += ms;
    r->windows++;
    if (err & 2) return th_fail(ctx, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
    if (!(err & 1)) return TH_OK;
    int mx = 0;
    for (int i = first; i <= n; ++i) mx = std::max(mx, cnt[i]);
    r->slot_cap = ((mx + 256) / 32 + 1) * 32;
    th_status st2 = alloc_window(ctx, r, r->win_slots, r->slot_cap);
    if (st2 != TH_OK) return st2;
  }
  return th_fail(ctx, TH_ERR_CAPACITY, "node window growth did not converge");
}

th_status read_counters(th_ctx* ctx, RunState* r, TrackCounters* h) {
  th_status st = th_cuda_check(ctx, cudaMemcpyAsync(h, r->S.C, sizeof(TrackCounters), cudaMemcpyDeviceToHost,
                                                    ctx->stream), "copy");
  if (st != TH_OK) return st;
  int err = 0;
  st = th_cuda_check(ctx, cudaMemcpyAsync(&err, r->S.err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "copy");
  if (st != TH_OK) return st;
  st = th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "solidification step");
  if (st != TH_OK) return st;
  if (err & 16) {
    char b[256];
    std::snprintf(b, sizeof(b), "a %s wait exceeded its limit (step %d, ticket %d, initial items %d, tickets %d, "
                  "published %d, published %d, completed %d, errors 0x%x)", h->diag[0] == 2 ? "grid barrier" : "work-queue",
                  h->diag[1], h->diag[2], h->diag[3], h->diag[4], h->diag[5], h->diag[6], h->diag[7], err);
    return th_fail(ctx, TH_ERR_TIMEOUT, b);
  }
  if (err & 32) return th_fail(ctx, TH_ERR_CAPACITY, "solidification record queue overflowed");
  if (err & 64) return th_fail(ctx, TH_ERR_CAPACITY, "a tracking list overflowed");
  if (err & 128) return th_fail(ctx, TH_ERR_CAPACITY, "the per-step work queue overflowed");
  if (err & 2) return th_fail(ctx, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
  return TH_OK;
}

th_status drain_records(th_ctx* ctx, RunState* r, int nrec) {
  if (nrec <= 0) return TH_OK;
  th_launch_solidify(ctx->dp, r->S, std::min(nrec, r->S.rec_cap), ctx->precision, ctx->hp.do_sol, ctx->stream);
  th_status st = th_cuda_check(ctx, cudaGetLastError(), "solidify");
  if (st != TH_OK) return st;
  return th_cuda_check(ctx, cudaMemsetAsync(&r->S.C->rec_n, 0, sizeof(int), ctx->stream), "cudaMemsetAsync");
}

// Advances the solidification loop until it finishes, reaches step `stop_at` (exclusive)
// or max_steps.
th_status advance(th_ctx* ctx, int64_t stop_at) {
  RunState* r = ctx->run;
  const HostProblem& hp = ctx->hp;
  const bool track = hp.tracking != TH_TRACK_NONE;
  const int window = track ? kWindowTrack : kWindowNoTrack;
  std::vector<double> ts;
  while (!r->done && r->k < stop_at) {
    const int n = (int)std::min<int64_t>(window, stop_at - r->k);
    th_status st = build_window(ctx, r, n, ts);
    if (st != TH_OK) return st;
    TrackCounters h;
    cudaEventRecord(r->ev[0], ctx->stream);
    if (track) {
      st = th_cuda_check(ctx, cudaMemsetAsync(r->S.bar, 0, 2 * sizeof(unsigned), ctx->stream), "cudaMemsetAsync");
      if (st != TH_OK) return st;
      st = th_cuda_check(ctx, th_launch_track(ctx->dp, r->S, r->W, r->k, r->k + n, ctx->precision, r->S.rec_cap / 2,
                                              ctx->stream), "cooperative launch");
      if (st != TH_OK) return st;
    } else {
      for (int k = r->k; k < r->k + n; ++k) th_launch_notrack_step(ctx->dp, r->S, r->W, k, ctx->precision, ctx->stream);
      st = th_cuda_check(ctx, cudaGetLastError(), "notrack step");
      if (st != TH_OK) return st;
    }
    cudaEventRecord(r->ev[1], ctx->stream);
    st = read_counters(ctx, r, &h);
    if (st != TH_OK) return st;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r->ev[0], r->ev[1]);
    r->ms_track += ms;
    cudaEventRecord(r->ev[0], ctx->stream);
    st = drain_records(ctx, r, h.rec_n);
    if (st != TH_OK) return st;
    cudaEventRecord(r->ev[1], ctx->stream);
    r->records += h.rec_n;
    const int k_new = h.step;
    if (k_new <= r->k && !h.done) return th_fail(ctx, TH_ERR_INVALID, "solidification loop made no progress");
    // times of the steps actually run (slots are 1-based from r->k)
    const int ran = k_new - r->k;
    r->t_prev = ts[ran];
    r->t_next = ran + 1 <= n ? ts[ran + 1] : ts[n] + hp.dt;
    r->k = k_new;
    r->done = h.done != 0;
    cudaEventSynchronize(r->ev[1]);
    cudaEventElapsedTime(&ms, r->ev[0], r->ev[1]);
    r->ms_solid += ms;
    r->max_rounds = std::max(r->max_rounds, h.max_items);
  }
  return th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "solidification");
}

int field_id(const std::string& f) {
  static const char* names[] = {"T", "tSol", "G", "V", "Gx", "Gy", "Gz", "dTdt", "eqFrac", "numMelt", "depth", "output_flag"};
  for (int i = 0; i < 12; ++i) if (f == names[i]) return i;
  return -1;
}

th_status fetch_field(th_ctx* ctx, int id, double* out) {
  RunState* r = ctx->run;
  th_status st = TH_OK;
  if (!r->d_field) {
    st = th_cuda_check(ctx, cudaMalloc(&r->d_field, ctx->hp.pnum * sizeof(double)), "cudaMalloc");
    if (st != TH_OK) return st;
  }
  th_launch_final_field(ctx->dp, r->S, id, r->d_field, ctx->stream);
  st = th_cuda_check(ctx, cudaGetLastError(), "field");
  if (st != TH_OK) return st;
  st = th_cuda_check(ctx, cudaMemcpyAsync(out, r->d_field, ctx->hp.pnum * sizeof(double), cudaMemcpyDeviceToHost,
                                          ctx->stream), "cudaMemcpyAsync");
  if (st != TH_OK) return st;
  return th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "field");
}

th_status write_solidification_csv(th_ctx* ctx, const std::string& tag) {
  const HostProblem& hp = ctx->hp;
  const int64_t n = hp.pnum;
  std::vector<double> x, y, z;
  th_grid_coords(hp, x, y, z);
  std::vector<std::string> names;
  std::vector<std::vector<double>> store;
  std::vector<const double*> cols;
  auto add = [&](bool on, const char* nm, int id) -> th_status {
    if (!on) return TH_OK;
    store.emplace_back(n);
    th_status st = fetch_field(ctx, id, store.back().data());
    names.push_back(nm);
    return st;
  };
  th_status st;
  if ((st = add(hp.o_T, "T", F_T)) != TH_OK) return st;
  if ((st = add(hp.o_tSol, "tSol", F_TSOL)) != TH_OK) return st;
  if ((st = add(hp.o_G, "G", F_G)) != TH_OK) return st;
  if ((st = add(hp.o_V, "V", F_V)) != TH_OK) return st;
  if ((st = add(hp.o_Gx, "Gx", F_GX)) != TH_OK) return st;
  if ((st = add(hp.o_Gy, "Gy", F_GY)) != TH_OK) return st;
  if ((st = add(hp.o_Gz, "Gz", F_GZ)) != TH_OK) return st;
  if ((st = add(hp.o_dTdt, "dTdt", F_DTDT)) != TH_OK) return st;
  if ((st = add(hp.o_eqFrac, "eqFrac", F_EQ)) != TH_OK) return st;
  if ((st = add(hp.o_depth && hp.tracking == TH_TRACK_SURFACE, "depth", F_DEPTH)) != TH_OK) return st;
  if ((st = add(hp.o_numMelt, "numMelt", F_NUMMELT)) != TH_OK) return st;
  std::vector<double> flagd(n);
  if ((st = fetch_field(ctx, F_FLAG, flagd.data())) != TH_OK) return st;
  std::vector<unsigned char> flag(n);
  for (int64_t p = 0; p < n; ++p) flag[p] = flagd[p] != 0.0;
  std::vector<std::string> all;
  std::vector<const double*> allc;
  if (hp.o_x) { all.push_back("x"); allc.push_back(x.data()); }
  if (hp.o_y) { all.push_back("y"); allc.push_back(y.data()); }
  if (hp.o_z) { all.push_back("z"); allc.push_back(z.data()); }
  for (size_t i = 0; i < names.size(); ++i) { all.push_back(names[i]); allc.push_back(store[i].data()); }
  std::string err;
  if (!th_write_csv(hp, tag, all, allc, flag.data(), err)) return th_fail(ctx, TH_ERR_IO, err);
  return TH_OK;
}

}  // namespace

extern "C" {

th_status th_solidify(th_ctx* ctx, int64_t max_steps, int64_t* steps_out) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  if (ctx->hp.mode != 1) return th_fail(ctx, TH_ERR_INVALID, "the deck is not a Solidification deck");
  th_status st = th_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (st != TH_OK) return st;
  if (!ctx->run) {
    st = init_run(ctx);
    if (st != TH_OK) return st;
  }
  const int64_t stop = max_steps > 0 ? std::min<int64_t>(max_steps, INT_MAX - 1) : (int64_t)INT_MAX - 1;
  RunState* r = ctx->run;
  cudaEventRecord(r->ev_run[0], ctx->stream);
  st = advance(ctx, stop);
  cudaEventRecord(r->ev_run[1], ctx->stream);
  if (cudaEventSynchronize(r->ev_run[1]) == cudaSuccess) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r->ev_run[0], r->ev_run[1]);
    r->ms_device += ms;
  }
  if (steps_out) *steps_out = ctx->run->k;
  return st;
}

th_status th_run_reset(th_ctx* ctx) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  th_status st = th_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (st != TH_OK) return st;
  RunState* r = ctx->run;
  if (!r) return TH_OK;
  // the buffers stay allocated; every one is refilled with its initial contents
  for (size_t i = 0; i < r->allocs.size(); ++i) {
    st = th_cuda_check(ctx, cudaMemsetAsync(r->allocs[i], r->alloc_fill[i].second, r->alloc_fill[i].first, ctx->stream),
                       "cudaMemsetAsync");
    if (st != TH_OK) return st;
  }
  if (ctx->hp.tracking == TH_TRACK_NONE) k_fill_d<<<1024, 256, 0, ctx->stream>>>(r->S.T, (int64_t)ctx->hp.pnum, ctx->hp.T0);
  r->k = 0; r->t_prev = 0.0; r->t_next = 0.0; r->done = false; r->max_rounds = 0;
  r->ms_nodes = r->ms_track = r->ms_solid = r->ms_device = 0;
  r->windows = r->records = 0;
  st = th_cuda_check(ctx, cudaMemsetAsync(ctx->d_pairs, 0, 2 * sizeof(unsigned long long), ctx->stream), "cudaMemsetAsync");
  if (st != TH_OK) return st;
  return th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "reset");
}

th_status th_run_stats(th_ctx* ctx, double* out, int32_t n) {
  if (!ctx || !out) return th_fail(ctx, TH_ERR_INVALID, "null argument");
  const RunState* r = ctx->run;
  unsigned long long pairs[2] = {0, 0};
  th_status st = th_cuda_check(ctx, cudaMemcpy(pairs, ctx->d_pairs, sizeof(pairs), cudaMemcpyDeviceToHost), "cudaMemcpy");
  if (st != TH_OK) return st;
  const double v[11] = {r ? r->ms_nodes : 0, r ? r->ms_track : 0, r ? r->ms_solid : 0, r ? (double)r->windows : 0,
                        r ? (double)r->records : 0, r ? (double)r->max_rounds : 0, r ? (double)r->k : 0,
                        r ? (double)r->slot_cap : 0, r ? r->ms_device : 0, (double)pairs[1],
                        (double)pairs[0]};
  for (int i = 0; i < n && i < 11; ++i) out[i] = v[i];
  return TH_OK;
}

th_status th_field(th_ctx* ctx, const char* name, double* out) {
  if (!ctx || !name || !out) return th_fail(ctx, TH_ERR_INVALID, "null argument");
  th_status st = th_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (st != TH_OK) return st;
  const std::string f(name);
  const int64_t n = ctx->hp.pnum;
  if (ctx->hp.mode == 0) {
    if (f == "T") {
      if (!ctx->T_valid) return th_fail(ctx, TH_ERR_INVALID, "no temperature field computed yet");
      return th_cuda_check(ctx, cudaMemcpy(out, ctx->d_T, n * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy");
    }
    if (f == "output_flag") {
      for (int64_t p = 0; p < n; ++p) out[p] = 1.0;
      return TH_OK;
    }
    return th_fail(ctx, TH_ERR_INVALID, "field " + f + " is not available in Snapshots mode");
  }
  if (!ctx->run) return th_fail(ctx, TH_ERR_INVALID, "run th_solidify first");
  const int id = field_id(f);
  if (id < 0) return th_fail(ctx, TH_ERR_INVALID, "unknown field " + f);
  return fetch_field(ctx, id, out);
}

th_status th_simulate(th_ctx* ctx) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  const HostProblem& hp = ctx->hp;
  if (hp.mode == 0) {
    // Snapshots, Tracking None (src/Run.cpp:80-124): every point is output
    std::vector<double> x, y, z, T(hp.pnum);
    th_grid_coords(hp, x, y, z);
    std::vector<std::string> names;
    std::vector<const double*> cols;
    if (hp.o_x) { names.push_back("x"); cols.push_back(x.data()); }
    if (hp.o_y) { names.push_back("y"); cols.push_back(y.data()); }
    if (hp.o_z) { names.push_back("z"); cols.push_back(z.data()); }
    if (hp.o_T) { names.push_back("T"); cols.push_back(T.data()); }
    for (int i = 0; i < (int)hp.snaps.size(); ++i) {
      th_status st = th_snapshot(ctx, i, T.data());
      if (st != TH_OK) return st;
      std::string err;
      if (!th_write_csv(hp, "Snapshot." + th_zero_pad(i, 2), names, cols, nullptr, err))
        return th_fail(ctx, TH_ERR_IO, err);
    }
    return TH_OK;
  }
  th_status st = th_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (st != TH_OK) return st;
  if (!ctx->run && (st = init_run(ctx)) != TH_OK) return st;
  // intermediate outputs every OutputFrequency steps (src/Run.cpp:446-458, 553-565, 689-701)
  const std::string prefix = hp.tracking == TH_TRACK_SURFACE ? "Solidification." : "";
  const int64_t freq = hp.out_freq;
  while (!ctx->run->done) {
    int64_t stop = (int64_t)INT_MAX - 1;
    if (freq != INT_MAX && freq > 0) stop = (ctx->run->k / freq + 1) * freq + 1;   // run through step k*freq
    if ((st = advance(ctx, stop)) != TH_OK) return st;
    const int64_t last = ctx->run->k - 1;
    if (ctx->run->done) {
      if (freq != INT_MAX && freq > 0 && last > 0 && last % freq == 0)
        if ((st = write_solidification_csv(ctx, prefix + th_zero_pad((int)last, 7))) != TH_OK) return st;
      if (freq != INT_MAX && freq > 0) {
        const int64_t it = (last / freq + 1) * freq;
        if ((st = write_solidification_csv(ctx, prefix + th_zero_pad((int)it, 7))) != TH_OK) return st;
      }
      break;
    }
    if (freq != INT_MAX && freq > 0 && last > 0 && last % freq == 0)
      if ((st = write_solidification_csv(ctx, prefix + th_zero_pad((int)last, 7))) != TH_OK) return st;
  }
  return write_solidification_csv(ctx, "Solidification.Final");
}

}  // extern "C"
