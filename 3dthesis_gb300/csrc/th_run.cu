// Mode drivers behind th_simulate / th_solidify / th_field.
//
// Solidification (src/Run.cpp:390-709) runs in windows of steps.  The host lays out the
// step times exactly as the reference accumulates them (t += dt); one kernel builds a
// window's node lists (one warp per step); the persistent tracking kernel (Volume /
// Surface) or one whole-grid kernel per step (NoTracking) advances the state; and the
// queued liquid -> solid records are solidified in bulk.  For the tracking modes the three
// overlap: while the tracking kernel runs window w on the context's stream, a second
// stream builds the node lists of window w + 1 and solidifies the records of window w - 1
// (two node windows and two record buffers, ordered by events).  Stork logs each launch's
// liquid lists instead of records; the aux stream turns a finished launch's log into the
// doubly reduced data while the next launch runs.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "th_ctx.h"
#include "th_output.h"
#include "th_track.h"

namespace {

enum { F_T, F_TSOL, F_G, F_V, F_GX, F_GY, F_GZ, F_DTDT, F_EQ, F_NUMMELT, F_DEPTH, F_FLAG };

constexpr int kWindowTrack = 256;     // steps per node window (tracking)
constexpr int kWindowNoTrack = 32;    // steps per node window (NoTracking: whole grid per step)
constexpr int kRecCap = 1 << 22;      // solidification records per buffer
constexpr int kRedoListCap = 4096;    // nodes of each FP64 redo block's scratch list (longer lists: warp path)

struct Window {
  void* mem = nullptr;
  NodeWindow W{};
  double* d_t = nullptr;
  int* d_count = nullptr;
  int* d_seeds = nullptr;
  int* d_nseed = nullptr;
  int slots = 0;
  int base = 0, n = 0;                // steps [base, base + n) in slots 1..n
  cudaEvent_t gen0 = nullptr, gen1 = nullptr;   // around the node build
};

}  // namespace

struct RunState {
  TrackState S{};
  std::vector<void*> allocs;
  std::vector<std::pair<size_t, int>> alloc_fill;   // bytes and fill byte of each allocation
  Window win[2];
  SolRec* rec[2] = {nullptr, nullptr};
  int slot_cap = 1024;
  int seed_cap = 256;     // beam-trace candidates per step
  int k = 0;              // next step
  std::vector<double> times;   // step times, accumulated as the reference does
  bool done = false;
  bool initialised = false;
  int max_items = 0;
  double* d_field = nullptr;
  float2* d_axis = nullptr;
  cudaStream_t aux = nullptr;
  int* h_err = nullptr;        // pinned: node-build error bits per window
  cudaEvent_t ev_trk[2][2] = {};  // around each window's tracking launch
  cudaEvent_t ev_sol[2][2] = {};  // around each record buffer's solidification
  bool sol_timed[2] = {true, true};  // the events of ev_sol[b] have been added to ms_solid
  cudaEvent_t ev_run[2] = {nullptr, nullptr};
  double ms_nodes = 0, ms_track = 0, ms_solid = 0, ms_device = 0;
  long long windows = 0, records = 0;
  // Stork: per buffer the launch's log of liquid lists and their offsets, the launch's first
  // step and steps run (0: nothing pending); the rows on the device and their capacity
  int2* rlog[2] = {nullptr, nullptr};
  int* rlog_off[2] = {nullptr, nullptr};
  int rr_k0[2] = {0, 0}, rr_n[2] = {0, 0};
  int* h_off = nullptr;          // pinned: one log's offsets
  int* h_counts = nullptr;       // pinned: per step rows, vertex values
  long long* h_row_base = nullptr;   // pinned
  int* d_counts = nullptr;
  long long* d_row_base = nullptr;
  int* d_rerr = nullptr;
  int* d_rscratch = nullptr;
  size_t rscratch_ints = 0;
  double* d_rvals = nullptr;
  size_t rvals_doubles = 0;
  uint32_t* r_idx = nullptr;
  double* r_ts = nullptr;
  double* r_Ts = nullptr;
  long long rows = 0, rows_cap = 0;
  cudaEvent_t ev_rr[2] = {nullptr, nullptr};   // around the latest pass
  bool rr_timed = true;
  double ms_rrdf = 0;
  // RDF: the melt-event logs of the two launch buffers (Surface runs) and the events of the
  // run so far, every record's solidification time and cooling rate, all on the device
  int2* tm_log[2] = {nullptr, nullptr};
  int pending_tm[2] = {0, 0};
  int2* tm_all = nullptr;
  long long tm_total = 0, tm_all_cap = 0;
  RdfSol* rdf_sol = nullptr;
  long long rdf_total = 0, rdf_sol_cap = 0;
};

void th_release_run_state(th_ctx* ctx) {
  RunState* r = ctx->run;
  if (!r) return;
  if (r->aux) cudaStreamSynchronize(r->aux);
  for (void* p : r->allocs) cudaFree(p);
  for (Window& w : r->win) {
    cudaFree(w.mem); cudaFree(w.d_t); cudaFree(w.d_count); cudaFree(w.d_seeds); cudaFree(w.d_nseed);
    if (w.gen0) cudaEventDestroy(w.gen0);
    if (w.gen1) cudaEventDestroy(w.gen1);
  }
  cudaFree(r->d_field);
  cudaFree(r->d_axis);
  if (r->h_err) cudaFreeHost(r->h_err);
  if (r->h_off) cudaFreeHost(r->h_off);
  if (r->h_counts) cudaFreeHost(r->h_counts);
  if (r->h_row_base) cudaFreeHost(r->h_row_base);
  cudaFree(r->d_rscratch); cudaFree(r->d_rvals);
  cudaFree(r->r_idx); cudaFree(r->r_ts); cudaFree(r->r_Ts);
  cudaFree(r->tm_all); cudaFree(r->rdf_sol);
  for (int e = 0; e < 2; ++e) if (r->ev_rr[e]) cudaEventDestroy(r->ev_rr[e]);
  for (int b = 0; b < 2; ++b)
    for (int e = 0; e < 2; ++e) {
      if (r->ev_trk[b][e]) cudaEventDestroy(r->ev_trk[b][e]);
      if (r->ev_sol[b][e]) cudaEventDestroy(r->ev_sol[b][e]);
    }
  if (r->ev_run[0]) cudaEventDestroy(r->ev_run[0]);
  if (r->ev_run[1]) cudaEventDestroy(r->ev_run[1]);
  if (r->aux) cudaStreamDestroy(r->aux);
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

double time_of(RunState* r, double dt, int k) {
  while ((int)r->times.size() <= k) {
    if (r->times.empty()) r->times.push_back(0.0);
    else r->times.push_back(r->times.back() + dt);
  }
  return r->times[k];
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
  if (hp.tracking == TH_TRACK_NONE) ALLOC(S.T_last, n, 0);
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
    ALLOC(S.depth_max, ncol, 0);
  }
  if (hp.tracking == TH_TRACK_SURFACE || hp.tracking == TH_TRACK_STORK) ALLOC(S.depths, ncol, 0);
  const bool stork = hp.tracking == TH_TRACK_STORK;
  if (stork) {
    // a log holds the lists of one launch (a list has at most one entry per column); the
    // launch stops before less than one list's room is left
    S.rlog_step_max = (int)std::min<size_t>(ncol, (size_t)INT_MAX / 4);
    S.rlog_cap = (int)std::min<size_t>(std::max<size_t>((size_t)1 << 20, 4 * ncol), (size_t)INT_MAX / 2);
    for (int b = 0; b < 2; ++b) {
      ALLOC(r->rlog[b], (size_t)S.rlog_cap, 0);
      ALLOC(r->rlog_off[b], (size_t)kWindowTrack + 2, 0);
    }
    ALLOC(r->d_counts, 2 * (size_t)kWindowTrack, 0);
    ALLOC(r->d_row_base, (size_t)kWindowTrack, 0);
    ALLOC(r->d_rerr, 1, 0);
  }
  if (hp.tracking != TH_TRACK_NONE) {
    // the step word's fields bound a step's items (2^24 - 1 for Volume, 2^18 - 1 for the
    // Surface forms) and the Surface forms' liquid points (2^18 - 1: their lists hold
    // surface points only)
    const bool vol = hp.tracking == TH_TRACK_VOLUME;
    const size_t field = vol ? ((size_t)1 << 24) - 1 : ((size_t)1 << 18) - 1;
    S.list_cap = (int)(vol ? n : std::min<size_t>(n, field));
    for (int i = 0; i < 3; ++i) ALLOC(S.liq[i], n, 0);
    // work items of one step: every claimed point and column layer at most once, which
    // in practice stays far below 2 * pnum
    S.queue_cap = (int)std::min<size_t>(2 * n + 4096, field);
    // test knob of the failure path: a smaller work queue overflows (ERR_QUEUE)
    if (const char* env = std::getenv("THESIS_GB300_QUEUE_CAP")) {
      const int v = std::atoi(env);
      if (v > 0) S.queue_cap = std::min(S.queue_cap, v);
    }
    ALLOC(S.queue, (size_t)S.queue_cap, 0);
  }
  if (hp.o_rdf && hp.tracking == TH_TRACK_SURFACE) {   // melt events (only Surface's reset sweep opens them)
    ALLOC(S.rdf_open, n, 0);
    S.tm_cap = 1 << 20;
    ALLOC(r->tm_log[0], (size_t)S.tm_cap, 0);
    ALLOC(r->tm_log[1], (size_t)S.tm_cap, 0);
  }
  // Stork queues no records: its buffers stay token-sized
  const int rec_alloc = stork ? 64 : kRecCap;
  S.rec_cap = rec_alloc;
  // test knob of the failure path: record buffers this small overflow in one step (ERR_RECORDS)
  if (const char* env = std::getenv("THESIS_GB300_REC_CAP")) {
    const int v = std::atoi(env);
    if (v > 0) S.rec_cap = std::min(S.rec_cap, v);
  }
  ALLOC(r->rec[0], (size_t)rec_alloc, 0);
  ALLOC(r->rec[1], (size_t)rec_alloc, 0);
  // the FP64 redo of FP32 solidification (queue, scratch lists); compressing decks
  // solidify every record with the same kernel
  if (ctx->precision == TH_FP32_KAHAN || hp.compress) {
    ALLOC(S.redo, (size_t)kRecCap, 0);
    ALLOC(S.redo_n, 1, 0);
    ALLOC(S.fix, (size_t)kRecCap, 0);
    ALLOC(S.fix_n, 1, 0);
    ALLOC(S.fix_T, (size_t)kRecCap, 0);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    S.redo_blocks = std::max(1, sms);
    S.redo_cap = kRedoListCap;
    const size_t cap = (size_t)S.redo_blocks * S.redo_cap;
    double* d = nullptr;
    ALLOC(d, cap * 13, 0);                      // 8 double and 10 float fields per node
    float* f = (float*)(d + 8 * cap);
    NodeBufView& nb = S.redo_nb;
    nb.cap = (int)cap;
    nb.x = d; nb.y = d + cap; nb.z = d + 2 * cap; nb.ipx = d + 3 * cap; nb.ipy = d + 4 * cap; nb.ipz = d + 5 * cap;
    nb.dtau = d + 6 * cap; nb.amp = d + 7 * cap;
    nb.kx = f; nb.ky = f + cap; nb.kz = f + 2 * cap; nb.w = f + 3 * cap; nb.xh = f + 4 * cap; nb.xl = f + 5 * cap;
    nb.yh = f + 6 * cap; nb.yl = f + 7 * cap; nb.zh = f + 8 * cap; nb.zl = f + 9 * cap;
    ALLOC(S.redo_aux, 2 * (size_t)S.redo_blocks, 0);
  }
  ALLOC(S.C, 1, 0);
  ALLOC(S.err, 1, 0);
#undef ALLOC
  {  // point coordinates (the device's coord(): min + i * h, or max on a one-point axis) as float pairs
    const DevProblem& D = ctx->dp;
    std::vector<float2> ax;
    auto axis = [&](int g, int cnt, double vmin, double vmax, double h) {
      for (int i = 0; i < cnt; ++i) {
        const double v = (g - 1) ? vmin + (double)i * h : vmax;
        const float hi = (float)v;
        ax.push_back(make_float2(hi, (float)(v - (double)hi)));
      }
    };
    axis(D.gx, D.nx, D.xmin, D.xmax, D.hx);
    axis(D.gy, D.ny, D.ymin, D.ymax, D.hy);
    axis(D.gz, D.nz, D.zmin, D.zmax, D.hz);
    if ((st = th_cuda_check(ctx, cudaMalloc(&r->d_axis, ax.size() * sizeof(float2)), "cudaMalloc")) != TH_OK) return st;
    if ((st = th_cuda_check(ctx, cudaMemcpy(r->d_axis, ax.data(), ax.size() * sizeof(float2), cudaMemcpyHostToDevice),
                            "copy")) != TH_OK)
      return st;
    S.axis = r->d_axis;
    S.t_fixed = (ctx->precision == TH_FP32_KAHAN && hp.tracking != TH_TRACK_NONE) ? 1 : 0;
  }
  S.pairs = ctx->d_pairs;
  S.rec = r->rec[0];
  S.rec_n = &S.C->rec_n[0];
  if (hp.tracking == TH_TRACK_NONE) {                 // NoTracking starts every point at T_0
    k_fill_d<<<1024, 256, 0, ctx->stream>>>(S.T, (int64_t)n, hp.T0);
    st = th_cuda_check(ctx, cudaGetLastError(), "fill");
    if (st != TH_OK) return st;
  }
  if ((st = th_cuda_check(ctx, cudaStreamCreateWithFlags(&r->aux, cudaStreamNonBlocking), "stream")) != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaHostAlloc((void**)&r->h_err, 4 * sizeof(int), cudaHostAllocDefault), "host")) != TH_OK)
    return st;
  if (stork) {
    if ((st = th_cuda_check(ctx, cudaHostAlloc((void**)&r->h_off, (kWindowTrack + 2) * sizeof(int), cudaHostAllocDefault),
                            "host")) != TH_OK)
      return st;
    if ((st = th_cuda_check(ctx, cudaHostAlloc((void**)&r->h_counts, 2 * kWindowTrack * sizeof(int), cudaHostAllocDefault),
                            "host")) != TH_OK)
      return st;
    if ((st = th_cuda_check(ctx, cudaHostAlloc((void**)&r->h_row_base, kWindowTrack * sizeof(long long),
                                               cudaHostAllocDefault), "host")) != TH_OK)
      return st;
    cudaEventCreate(&r->ev_rr[0]);
    cudaEventCreate(&r->ev_rr[1]);
  }
  for (int b = 0; b < 2; ++b) {
    cudaEventCreate(&r->win[b].gen0); cudaEventCreate(&r->win[b].gen1);
    for (int e = 0; e < 2; ++e) { cudaEventCreate(&r->ev_trk[b][e]); cudaEventCreate(&r->ev_sol[b][e]); }
  }
  cudaEventCreate(&r->ev_run[0]);
  cudaEventCreate(&r->ev_run[1]);
  r->k = 0;
  r->initialised = true;
  return th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "init");
}

th_status alloc_window(th_ctx* ctx, Window& w, int slots, int slot_cap, int seed_cap) {
  cudaFree(w.mem); w.mem = nullptr;
  cudaFree(w.d_t); w.d_t = nullptr;
  cudaFree(w.d_count); w.d_count = nullptr;
  cudaFree(w.d_seeds); w.d_seeds = nullptr;
  cudaFree(w.d_nseed); w.d_nseed = nullptr;
  const size_t cap = (size_t)slots * slot_cap;
  th_status st = th_cuda_check(ctx, cudaMalloc(&w.mem, cap * (8 * sizeof(double) + 10 * sizeof(float))), "cudaMalloc");
  if (st != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaMalloc(&w.d_t, slots * sizeof(double)), "cudaMalloc")) != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaMalloc(&w.d_count, slots * sizeof(int)), "cudaMalloc")) != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaMalloc(&w.d_seeds, (size_t)slots * seed_cap * sizeof(int)), "cudaMalloc")) != TH_OK)
    return st;
  if ((st = th_cuda_check(ctx, cudaMalloc(&w.d_nseed, slots * sizeof(int)), "cudaMalloc")) != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaMemset(w.d_nseed, 0, slots * sizeof(int)), "cudaMemset")) != TH_OK) return st;
  double* d = (double*)w.mem;
  float* f = (float*)(d + 8 * cap);
  NodeBufView& nb = w.W.nb;
  nb.cap = (int)cap;
  nb.x = d; nb.y = d + cap; nb.z = d + 2 * cap; nb.ipx = d + 3 * cap; nb.ipy = d + 4 * cap; nb.ipz = d + 5 * cap;
  nb.dtau = d + 6 * cap; nb.amp = d + 7 * cap;
  nb.kx = f; nb.ky = f + cap; nb.kz = f + 2 * cap; nb.w = f + 3 * cap; nb.xh = f + 4 * cap; nb.xl = f + 5 * cap;
  nb.yh = f + 6 * cap; nb.yl = f + 7 * cap; nb.zh = f + 8 * cap; nb.zl = f + 9 * cap;
  w.W.slot_cap = slot_cap;
  w.W.nslots = slots;
  w.W.count = w.d_count;
  w.W.t = w.d_t;
  w.W.seeds = w.d_seeds;
  w.W.nseed = w.d_nseed;
  w.W.seed_cap = seed_cap;
  w.slots = slots;
  return TH_OK;
}

// Enqueues the node lists of steps [base, base + n) (slots 1..n) and of step base - 1
// (slot 0) into window b on `s`; the error bits land in h_err[b] when w.gen1 completes.
th_status enqueue_window(th_ctx* ctx, RunState* r, int b, int base, int n, cudaStream_t s) {
  Window& w = r->win[b];
  if (!w.mem || w.slots < n + 1 || w.W.slot_cap != r->slot_cap || w.W.seed_cap != r->seed_cap) {
    th_status st = alloc_window(ctx, w, std::max(n + 1, std::max(w.slots, kWindowTrack + 1)), r->slot_cap,
                                r->seed_cap);
    if (st != TH_OK) return st;
  }
  std::vector<double> ts(n + 1);
  ts[0] = base > 0 ? time_of(r, ctx->hp.dt, base - 1) : 0.0;
  for (int i = 1; i <= n; ++i) ts[i] = time_of(r, ctx->hp.dt, base + i - 1);
  w.base = base; w.n = n; w.W.base = base;
  th_status st = th_cuda_check(ctx, cudaMemcpyAsync(w.d_t, ts.data(), (n + 1) * sizeof(double), cudaMemcpyHostToDevice, s),
                               "cudaMemcpyAsync");
  if (st != TH_OK) return st;
  int* d_err = ctx->d_small + 2 + b;
  if ((st = th_cuda_check(ctx, cudaMemsetAsync(d_err, 0, sizeof(int), s), "cudaMemsetAsync")) != TH_OK) return st;
  const int first = base == 0 ? 1 : 0;
  cudaEventRecord(w.gen0, s);
  th_launch_nodes_window(ctx->dp, w.W, first, n + 1 - first, false, d_err, s);
  if ((st = th_cuda_check(ctx, cudaGetLastError(), "node window")) != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaMemcpyAsync(r->h_err + b, d_err, sizeof(int), cudaMemcpyDeviceToHost, s), "copy")) != TH_OK)
    return st;
  cudaEventRecord(w.gen1, s);
  r->windows++;
  return TH_OK;
}

// Waits for window b's node build; on a capacity overflow grows the slots and rebuilds it
// synchronously.  *ok is false when the build had to be redone.
th_status finish_window(th_ctx* ctx, RunState* r, int b) {
  Window& w = r->win[b];
  for (int attempt = 0; attempt < 4; ++attempt) {
    th_status st = th_cuda_check(ctx, cudaEventSynchronize(w.gen1), "node window");
    if (st != TH_OK) return st;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, w.gen0, w.gen1);
    r->ms_nodes += ms;
    const int err = r->h_err[b];
    if (err & 2) return th_fail(ctx, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
    if (!(err & (1 | ERR_SEED_CAPACITY))) return TH_OK;
    std::vector<int> cnt(w.n + 1), ns(w.n + 1);
    st = th_cuda_check(ctx, cudaMemcpy(cnt.data(), w.d_count, (w.n + 1) * sizeof(int), cudaMemcpyDeviceToHost), "copy");
    if (st != TH_OK) return st;
    st = th_cuda_check(ctx, cudaMemcpy(ns.data(), w.d_nseed, (w.n + 1) * sizeof(int), cudaMemcpyDeviceToHost), "copy");
    if (st != TH_OK) return st;
    int mx = 0, ms_ = 0;
    for (int i = (w.base == 0 ? 1 : 0); i <= w.n; ++i) { mx = std::max(mx, cnt[i]); ms_ = std::max(ms_, ns[i]); }
    if (err & 1) r->slot_cap = std::max(r->slot_cap, ((mx + 256) / 128 + 1) * 128);   // whole padded lists
    if (err & ERR_SEED_CAPACITY) r->seed_cap = std::max(r->seed_cap, ((ms_ + 64) / 32 + 1) * 32);
    // the other window may still be in use by the tracking stream or the aux stream
    cudaStreamSynchronize(r->aux);
    cudaStreamSynchronize(ctx->stream);
    if ((st = enqueue_window(ctx, r, b, w.base, w.n, r->aux)) != TH_OK) return st;
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
  // a capacity overflow first: a lost work item also leaves the step's waits to run out
  if (err & 32) return th_fail(ctx, TH_ERR_CAPACITY, "solidification record queue overflowed");
  if (err & 1) return th_fail(ctx, TH_ERR_CAPACITY, "a solidification node list exceeded its buffer");
  if (err & 64) return th_fail(ctx, TH_ERR_CAPACITY, "a tracking list overflowed");
  if (err & 256) return th_fail(ctx, TH_ERR_CAPACITY, "the RDF melt-event log overflowed");
  if (err & 128) return th_fail(ctx, TH_ERR_CAPACITY, "the per-step work queue overflowed");
  if (err & 16) {
    char b[256];
    std::snprintf(b, sizeof(b), "a work-queue wait exceeded its limit (step %d, ticket %d, initial items %d, "
                  "tickets taken %d, blocks entered %d, published %d, completed %d, errors 0x%x)",
                  h->diag[1], h->diag[2], h->diag[3], h->diag[4], h->diag[5], h->diag[6], h->diag[7], err);
    return th_fail(ctx, TH_ERR_TIMEOUT, b);
  }
  if (err & 2) return th_fail(ctx, TH_ERR_TIMEOUT, "quadrature walk exceeded its step limit");
  return TH_OK;
}

void add_elapsed(double& acc, cudaEvent_t a, cudaEvent_t b);

// Grows a device array to hold `need` elements, keeping the first `keep` (stream-ordered
// copy on s; the old array is freed after it).
template <class T>
th_status grow(th_ctx* ctx, T** p, size_t need, size_t keep, cudaStream_t s) {
  T* q = nullptr;
  th_status st = th_cuda_check(ctx, cudaMalloc(&q, std::max<size_t>(need, 1) * sizeof(T)), "cudaMalloc");
  if (st != TH_OK) return st;
  if (*p && keep) {
    st = th_cuda_check(ctx, cudaMemcpyAsync(q, *p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
    if (st != TH_OK) { cudaFree(q); return st; }
    cudaStreamSynchronize(s);
  }
  cudaFree(*p);
  *p = q;
  return TH_OK;
}

// Stork: the doubly reduced data of the launch that filled log b (its steps, the node lists
// of window b), appended to the rows on stream s.  The host reads the log's offsets and then
// the per-step counts on the way (s holds only this pass), so the rows land at offsets laid
// out in step order and the buffers grow before the fill.
th_status rrdf_buffer(th_ctx* ctx, RunState* r, int b, cudaStream_t s) {
  const int n = r->rr_n[b];
  r->rr_n[b] = 0;
  if (n <= 0) return TH_OK;
  th_status st = th_cuda_check(ctx, cudaMemcpyAsync(r->h_off, r->rlog_off[b], (n + 2) * sizeof(int), cudaMemcpyDeviceToHost,
                                                    s), "copy");
  if (st != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaStreamSynchronize(s), "rrdf")) != TH_OK) return st;
  if (!r->rr_timed) { add_elapsed(r->ms_rrdf, r->ev_rr[0], r->ev_rr[1]); r->rr_timed = true; }
  if (r->h_off[n + 1] == 0) return TH_OK;                          // no liquid in these steps
  if (r->h_off[n + 1] > r->S.rlog_cap) return th_fail(ctx, TH_ERR_CAPACITY, "the Stork liquid-list log overflowed");
  int nmax = 1;
  for (int j = 0; j < n; ++j) nmax = std::max(nmax, r->h_off[j + 2] - r->h_off[j]);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = std::min(n, 2 * std::max(sms, 1));
  const size_t per = th_rrdf_scratch_ints(nmax);
  if ((size_t)blocks * per > r->rscratch_ints) {
    if ((st = grow(ctx, &r->d_rscratch, (size_t)blocks * per, 0, s)) != TH_OK) return st;
    r->rscratch_ints = (size_t)blocks * per;
  }
  RrdfBatch B{};
  B.log = r->rlog[b]; B.off = r->rlog_off[b]; B.k0 = r->rr_k0[b]; B.nsteps = n; B.nmax = nmax;
  B.counts = r->d_counts; B.row_base = r->d_row_base; B.scratch = r->d_rscratch; B.err = r->d_rerr;
  B.pairs = ctx->d_pairs;
  cudaEventRecord(r->ev_rr[0], s);
  th_launch_rrdf(ctx->dp, r->win[b].W, B, false, ctx->precision, blocks, s);
  if ((st = th_cuda_check(ctx, cudaGetLastError(), "rrdf count")) != TH_OK) return st;
  st = th_cuda_check(ctx, cudaMemcpyAsync(r->h_counts, r->d_counts, 2 * n * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
  if (st != TH_OK) return st;
  if ((st = th_cuda_check(ctx, cudaStreamSynchronize(s), "rrdf count")) != TH_OK) return st;
  long long total = 0;
  int nv = 1;
  for (int j = 0; j < n; ++j) {
    r->h_row_base[j] = r->rows + total;
    total += r->h_counts[2 * j];
    nv = std::max(nv, r->h_counts[2 * j + 1]);
  }
  if (total == 0) { cudaEventRecord(r->ev_rr[1], s); r->rr_timed = false; return TH_OK; }
  if (r->rows + total > r->rows_cap) {
    const long long cap = std::max<long long>(r->rows + total, std::max<long long>(2 * r->rows_cap, 1 << 16));
    if ((st = grow(ctx, &r->r_idx, 3 * (size_t)cap, 3 * (size_t)r->rows, s)) != TH_OK) return st;
    if ((st = grow(ctx, &r->r_ts, 2 * (size_t)cap, 2 * (size_t)r->rows, s)) != TH_OK) return st;
    if ((st = grow(ctx, &r->r_Ts, 16 * (size_t)cap, 16 * (size_t)r->rows, s)) != TH_OK) return st;
    r->rows_cap = cap;
  }
  if ((size_t)blocks * 3 * nv > r->rvals_doubles) {
    const size_t need = (size_t)blocks * 3 * std::max(nv, 4096);
    if ((st = grow(ctx, &r->d_rvals, need, 0, s)) != TH_OK) return st;
    r->rvals_doubles = need;
  }
  B.vals = r->d_rvals;
  B.vals_cap = (int)(r->rvals_doubles / (3 * (size_t)blocks));
  B.idx = r->r_idx; B.ts = r->r_ts; B.Ts = r->r_Ts;
  st = th_cuda_check(ctx, cudaMemcpyAsync(r->d_row_base, r->h_row_base, n * sizeof(long long), cudaMemcpyHostToDevice, s),
                     "copy");
  if (st != TH_OK) return st;
  th_launch_rrdf(ctx->dp, r->win[b].W, B, true, ctx->precision, blocks, s);
  if ((st = th_cuda_check(ctx, cudaGetLastError(), "rrdf fill")) != TH_OK) return st;
  cudaEventRecord(r->ev_rr[1], s);
  r->rr_timed = false;
  r->rows += total;
  return TH_OK;
}

// Solidifies record buffer b (nrec records) on stream s, then empties it.  The previous
// use of the buffer's events has completed by then (the tracking launch in between waited
// for it), so its time is added first.
th_status solidify_buffer(th_ctx* ctx, RunState* r, int b, int nrec, cudaStream_t s) {
  if (!r->sol_timed[b]) { add_elapsed(r->ms_solid, r->ev_sol[b][0], r->ev_sol[b][1]); r->sol_timed[b] = true; }
  r->sol_timed[b] = false;
  cudaEventRecord(r->ev_sol[b][0], s);
  nrec = std::min(nrec, r->S.rec_cap);
  if (nrec > 0) {
    TrackState S = r->S;
    if (ctx->hp.o_rdf) {                  // RDF: every record's time and rate, at the run's record count
      if (r->rdf_total + nrec > r->rdf_sol_cap) {
        const long long cap = std::max<long long>(r->rdf_total + nrec, std::max<long long>(2 * r->rdf_sol_cap, 1 << 16));
        th_status st = grow(ctx, &r->rdf_sol, (size_t)cap, (size_t)r->rdf_total, s);
        if (st != TH_OK) return st;
        r->rdf_sol_cap = cap;
      }
      S.rdf_sol = r->rdf_sol;
      S.rdf_base = r->rdf_total;
      r->rdf_total += nrec;
    }
    th_launch_solidify(ctx->dp, S, r->win[b].W, r->rec[b], nrec, ctx->precision, ctx->hp.do_sol, s);
    th_status st = th_cuda_check(ctx, cudaGetLastError(), "solidify");
    if (st != TH_OK) return st;
  }
  th_status st = th_cuda_check(ctx, cudaMemsetAsync(&r->S.C->rec_n[b], 0, sizeof(int), s), "cudaMemsetAsync");
  if (st == TH_OK && r->tm_log[b] && r->pending_tm[b] > 0) {     // RDF: this launch's melt events
    const int m = std::min(r->pending_tm[b], r->S.tm_cap);
    if (r->tm_total + m > r->tm_all_cap) {
      const long long cap = std::max<long long>(r->tm_total + m, std::max<long long>(2 * r->tm_all_cap, 1 << 16));
      if ((st = grow(ctx, &r->tm_all, (size_t)cap, (size_t)r->tm_total, s)) != TH_OK) return st;
      r->tm_all_cap = cap;
    }
    st = th_cuda_check(ctx, cudaMemcpyAsync(r->tm_all + r->tm_total, r->tm_log[b], m * sizeof(int2), cudaMemcpyDeviceToDevice,
                                            s), "cudaMemcpyAsync");
    if (st != TH_OK) return st;
    r->tm_total += m;
    r->pending_tm[b] = 0;
    st = th_cuda_check(ctx, cudaMemsetAsync(&r->S.C->tm_n[b], 0, sizeof(int), s), "cudaMemsetAsync");
  }
  if (st == TH_OK && ctx->hp.tracking == TH_TRACK_STORK) st = rrdf_buffer(ctx, r, b, s);
  cudaEventRecord(r->ev_sol[b][1], s);
  r->records += nrec;
  return st;
}

void add_elapsed(double& acc, cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) acc += ms;
}

// Tracking modes: pipelined windows.
th_status advance_tracking(th_ctx* ctx, int64_t stop_at) {
  RunState* r = ctx->run;
  const HostProblem& hp = ctx->hp;
  cudaStream_t ts = ctx->stream, as = r->aux;
  int b = 0;
  int pending_rec[2] = {0, 0};
  bool pending_sol[2] = {false, false};
  int n0 = (int)std::min<int64_t>(kWindowTrack, stop_at - r->k);
  if (n0 <= 0 || r->done) return TH_OK;
  // a launch ends after the step that takes its record buffer past half full; test knob:
  // THESIS_GB300_REC_HIGH_WATER lowers that mark (launches then end early, full-size buffers)
  int high_water = r->S.rec_cap / 2;
  if (const char* env = std::getenv("THESIS_GB300_REC_HIGH_WATER")) {
    const int v = std::atoi(env);
    if (v > 0) high_water = std::min(high_water, v);
  }
  th_status st = enqueue_window(ctx, r, b, r->k, n0, as);
  if (st != TH_OK) return st;
  while (true) {
    if ((st = finish_window(ctx, r, b)) != TH_OK) return st;
    Window& w = r->win[b];
    // the tracking launch may reuse record buffer b only after its last solidification
    cudaStreamWaitEvent(ts, w.gen1, 0);
    if (pending_sol[b]) cudaStreamWaitEvent(ts, r->ev_sol[b][1], 0);
    TrackState S = r->S;
    S.rec = r->rec[b];
    S.rec_n = &r->S.C->rec_n[b];
    S.rlog = r->rlog[b];
    S.rlog_off = r->rlog_off[b];
    if (r->tm_log[b]) { S.tm_log = r->tm_log[b]; S.tm_n = &r->S.C->tm_n[b]; }
    cudaEventRecord(r->ev_trk[b][0], ts);
    st = th_cuda_check(ctx, th_launch_track(ctx->dp, S, w.W, w.base, w.base + w.n, ctx->precision, high_water, ts),
                       "cooperative launch");
    if (st != TH_OK) return st;
    cudaEventRecord(r->ev_trk[b][1], ts);
    // meanwhile, on the aux stream: solidify the previous window's records and build the
    // next window (its buffer was last read by the previous tracking launch)
    const int nb = b ^ 1;
    if (pending_rec[nb] > 0 || pending_sol[nb]) {
      cudaStreamWaitEvent(as, r->ev_trk[nb][1], 0);
      if ((st = solidify_buffer(ctx, r, nb, pending_rec[nb], as)) != TH_OK) return st;
      pending_rec[nb] = 0;
    }
    const int next_base = w.base + w.n;
    const int next_n = (int)std::min<int64_t>(kWindowTrack, stop_at - next_base);
    bool prefetched = false;
    if (next_n > 0) {
      cudaStreamWaitEvent(as, r->ev_trk[nb][1], 0);
      if ((st = enqueue_window(ctx, r, nb, next_base, next_n, as)) != TH_OK) return st;
      prefetched = true;
    }
    TrackCounters h;
    if ((st = read_counters(ctx, r, &h)) != TH_OK) return st;
    add_elapsed(r->ms_track, r->ev_trk[b][0], r->ev_trk[b][1]);
    pending_rec[b] = h.rec_n[b];
    pending_sol[b] = true;
    r->max_items = std::max(r->max_items, h.max_items);
    const int k_new = h.step;
    if (k_new <= r->k && !h.done) return th_fail(ctx, TH_ERR_INVALID, "solidification loop made no progress");
    r->rr_k0[b] = w.base;
    r->pending_tm[b] = h.tm_n[b];
    r->rr_n[b] = ctx->hp.tracking == TH_TRACK_STORK ? k_new - w.base : 0;
    r->k = k_new;
    r->done = h.done != 0;
    if (r->done || r->k >= stop_at) break;
    if (r->k != next_base || !prefetched) {
      // stopped early at the record high-water mark: rebuild the next window from here
      cudaStreamSynchronize(as);
      const int n = (int)std::min<int64_t>(kWindowTrack, stop_at - r->k);
      if ((st = enqueue_window(ctx, r, nb, r->k, n, as)) != TH_OK) return st;
    }
    b = nb;
  }
  // drain: both record buffers, then wait for both streams
  for (int i = 0; i < 2; ++i) {
    const int bb = b ^ 1 ^ i;       // the older buffer first
    if (pending_rec[bb] > 0 || r->rr_n[bb] > 0 || r->pending_tm[bb] > 0) {
      cudaStreamWaitEvent(as, r->ev_trk[bb][1], 0);
      if ((st = solidify_buffer(ctx, r, bb, pending_rec[bb], as)) != TH_OK) return st;
      pending_rec[bb] = 0;
    }
  }
  if ((st = th_cuda_check(ctx, cudaStreamSynchronize(as), "solidify")) != TH_OK) return st;
  for (int i = 0; i < 2; ++i)
    if (!r->sol_timed[i]) { add_elapsed(r->ms_solid, r->ev_sol[i][0], r->ev_sol[i][1]); r->sol_timed[i] = true; }
  if (!r->rr_timed) { add_elapsed(r->ms_rrdf, r->ev_rr[0], r->ev_rr[1]); r->rr_timed = true; }
  if (r->d_rerr) {
    int e = 0;
    if ((st = th_cuda_check(ctx, cudaMemcpy(&e, r->d_rerr, sizeof(int), cudaMemcpyDeviceToHost), "copy")) != TH_OK) return st;
    if (e) return th_fail(ctx, TH_ERR_CAPACITY, "a Stork step needed more vertex values than laid out");
  }
  return th_cuda_check(ctx, cudaStreamSynchronize(ts), "solidification");
}

// NoTracking: one whole-grid kernel per step, windows built and drained in sequence.
th_status fetch_field(th_ctx* ctx, int id, double* out);

// After step k of a run without tracking: if the step ran, its time and every point's T join
// the temperature history.
th_status record_T_hist(th_ctx* ctx, RunState* r, int k) {
  int step = 0;
  th_status st = th_cuda_check(ctx, cudaMemcpyAsync(&step, &r->S.C->step, sizeof(int), cudaMemcpyDeviceToHost,
                                                    ctx->stream), "cudaMemcpyAsync");
  if (st != TH_OK || (st = th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "T_hist")) != TH_OK) return st;
  if (step != k + 1) return TH_OK;
  const size_t n = (size_t)ctx->hp.pnum, at = ctx->hist_T.size();
  try {                                   // every step adds pnum values on the host
    ctx->hist_T.resize(at + n);
    ctx->hist_t.reserve(ctx->hist_t.size() + 1);
  } catch (const std::bad_alloc&) {
    return th_fail(ctx, TH_ERR_CAPACITY, "the T_hist history does not fit in host memory");
  }
  if ((st = fetch_field(ctx, F_T, ctx->hist_T.data() + at)) != TH_OK) return st;
  ctx->hist_t.push_back(time_of(r, ctx->hp.dt, k));
  return TH_OK;
}

th_status advance_notrack(th_ctx* ctx, int64_t stop_at) {
  RunState* r = ctx->run;
  while (!r->done && r->k < stop_at) {
    const int n = (int)std::min<int64_t>(kWindowNoTrack, stop_at - r->k);
    th_status st = enqueue_window(ctx, r, 0, r->k, n, ctx->stream);
    if (st != TH_OK) return st;
    if ((st = finish_window(ctx, r, 0)) != TH_OK) return st;
    TrackState S = r->S;
    cudaEventRecord(r->ev_trk[0][0], ctx->stream);
    for (int k = r->k; k < r->k + n; ++k) {
      th_launch_notrack_step(ctx->dp, S, r->win[0].W, k, ctx->precision, ctx->stream);
      // Output T_hist 1: every point's T joins the history at each step the loop ran
      // (src/Grid.cpp:300-304; the loop runs no step after the finish test passed)
      if (ctx->hp.o_T_hist && (st = record_T_hist(ctx, r, k)) != TH_OK) return st;
    }
    if ((st = th_cuda_check(ctx, cudaGetLastError(), "notrack step")) != TH_OK) return st;
    cudaEventRecord(r->ev_trk[0][1], ctx->stream);
    TrackCounters h;
    if ((st = read_counters(ctx, r, &h)) != TH_OK) return st;
    add_elapsed(r->ms_track, r->ev_trk[0][0], r->ev_trk[0][1]);
    if ((st = solidify_buffer(ctx, r, 0, h.rec_n[0], ctx->stream)) != TH_OK) return st;
    if ((st = th_cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "solidify")) != TH_OK) return st;
    add_elapsed(r->ms_solid, r->ev_sol[0][0], r->ev_sol[0][1]);
    r->sol_timed[0] = true;
    if (h.step <= r->k && !h.done) return th_fail(ctx, TH_ERR_INVALID, "solidification loop made no progress");
    r->k = h.step;
    r->done = h.done != 0;
  }
  return TH_OK;
}

th_status advance(th_ctx* ctx, int64_t stop_at) {
  return ctx->hp.tracking == TH_TRACK_NONE ? advance_notrack(ctx, stop_at) : advance_tracking(ctx, stop_at);
}

int field_id(const std::string& f) {
  static const char* names[] = {"T", "tSol", "G", "V", "Gx", "Gy", "Gz", "dTdt", "eqFrac", "numMelt", "depth", "output_flag"};
  for (int i = 0; i < 12; ++i) if (f == names[i]) return i;
  return -1;
}

// RDF: every point's melt events as the reference's Grid holds them (src/Grid.h:103-105,
// 360-362), sorted by point, then step: the melting times - events logged before the last
// step run, as t - dt of the step after them (the reference pushes them at the start of
// that step) - and every solidification's time and cooling rate.
struct RdfHost {
  std::vector<std::pair<int, double>> tm;   // (point, melting time)
  std::vector<RdfSol> sol;                  // (point, step, solidification time, cooling rate)
};

th_status gather_rdf(th_ctx* ctx, RdfHost& h) {
  RunState* r = ctx->run;
  std::vector<int2> ev((size_t)r->tm_total);
  h.sol.assign((size_t)r->rdf_total, RdfSol{});
  th_status st = TH_OK;
  if (!ev.empty() && (st = th_cuda_check(ctx, cudaMemcpy(ev.data(), r->tm_all, ev.size() * sizeof(int2),
                                                         cudaMemcpyDeviceToHost), "cudaMemcpy")) != TH_OK)
    return st;
  if (!h.sol.empty() && (st = th_cuda_check(ctx, cudaMemcpy(h.sol.data(), r->rdf_sol, h.sol.size() * sizeof(RdfSol),
                                                            cudaMemcpyDeviceToHost), "cudaMemcpy")) != TH_OK)
    return st;
  const int last = r->k - 1;
  std::sort(ev.begin(), ev.end(), [](const int2& a, const int2& b) { return a.x != b.x ? a.x < b.x : a.y < b.y; });
  h.tm.clear();
  for (const int2& e : ev)
    if (e.y < last) h.tm.push_back({e.x, time_of(r, ctx->hp.dt, e.y + 1) - ctx->hp.dt});
  std::sort(h.sol.begin(), h.sol.end(),
            [](const RdfSol& a, const RdfSol& b) { return a.p != b.p ? a.p < b.p : a.step < b.step; });
  return TH_OK;
}

th_status fetch_field(th_ctx* ctx, int id, double* out) {
  RunState* r = ctx->run;
  th_status st = TH_OK;
  if (id == F_NUMMELT && ctx->hp.o_rdf) {    // with RDF the count is the number of melting times (src/Grid.h:343-350)
    RdfHost h;
    if ((st = gather_rdf(ctx, h)) != TH_OK) return st;
    std::fill(out, out + ctx->hp.pnum, 0.0);
    for (const auto& e : h.tm) out[e.first] += 1.0;
    return TH_OK;
  }
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

// Grid::Output_RDF (src/Grid.cpp:176-201): per output point, per melting time, the point's
// coordinates, the melting time, and the solidification time and cooling rate of the same
// index.  Where a point has more melting than solidification times the reference reads past
// the end of its vectors; those rows get 0 here.
th_status write_rdf_csv(th_ctx* ctx, const std::string& tag) {
  RdfHost h;
  th_status st = gather_rdf(ctx, h);
  if (st != TH_OK) return st;
  std::vector<double> flagd(ctx->hp.pnum);
  if ((st = fetch_field(ctx, F_FLAG, flagd.data())) != TH_OK) return st;
  std::vector<int64_t> pts;
  std::vector<double> tm, tl, cr;
  size_t a = 0, b = 0;
  while (a < h.tm.size()) {
    const int p = h.tm[a].first;
    while (b < h.sol.size() && h.sol[b].p < p) ++b;
    size_t e = 0;
    for (; a < h.tm.size() && h.tm[a].first == p; ++a, ++e) {
      if (flagd[p] == 0.0) continue;
      const bool has = b + e < h.sol.size() && h.sol[b + e].p == p;
      pts.push_back(p);
      tm.push_back(h.tm[a].second);
      tl.push_back(has ? h.sol[b + e].tsol : 0.0);
      cr.push_back(has ? h.sol[b + e].cr : 0.0);
    }
  }
  std::string err;
  if (!th_write_rdf_csv(ctx->hp, tag, pts.data(), tm.data(), tl.data(), cr.data(), (int64_t)pts.size(), err))
    return th_fail(ctx, TH_ERR_IO, err);
  return TH_OK;
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
  r->k = 0; r->done = false; r->max_items = 0;
  ctx->hist_t.clear();
  ctx->hist_T.clear();
  r->sol_timed[0] = r->sol_timed[1] = true;
  r->ms_nodes = r->ms_track = r->ms_solid = r->ms_device = 0;
  r->rows = 0; r->rr_n[0] = r->rr_n[1] = 0; r->rr_timed = true; r->ms_rrdf = 0;
  r->tm_total = 0; r->rdf_total = 0; r->pending_tm[0] = r->pending_tm[1] = 0;
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
  unsigned long long prof[21] = {};     // the loop profile, then the FP64 redo, guard and fix counts
  if (r && r->S.C) {
    st = th_cuda_check(ctx, cudaMemcpy(prof, r->S.C->prof, sizeof(prof), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (st != TH_OK) return st;
  }
  const double v[34] = {r ? r->ms_nodes : 0, r ? r->ms_track : 0, r ? r->ms_solid : 0, r ? (double)r->windows : 0,
                        r ? (double)r->records : 0, r ? (double)r->max_items : 0, r ? (double)r->k : 0,
                        r ? (double)r->slot_cap : 0, r ? r->ms_device : 0, (double)pairs[1],
                        (double)pairs[0], prof[0] * 1e-6, prof[1] * 1e-6, (double)prof[2], (double)prof[3],
                        (double)prof[4], (double)prof[5], (double)prof[6], (double)prof[7], (double)prof[8],
                        prof[10] * 1e-6, prof[11] * 1e-6, prof[12] * 1e-6, prof[13] * 1e-6,
                        prof[14] * 1e-6, prof[15] * 1e-6, prof[16] * 1e-6, prof[17] * 1e-6,
                        (double)prof[9], (double)prof[18], (double)prof[19],
                        r ? r->ms_rrdf : 0, r ? (double)r->rows : 0, (double)prof[20]};
  for (int i = 0; i < n && i < 34; ++i) out[i] = v[i];
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

th_status th_rrdf(th_ctx* ctx, uint32_t* idx, double* ts, double* Ts, int64_t cap, int64_t* rows) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  if (ctx->hp.tracking != TH_TRACK_STORK) return th_fail(ctx, TH_ERR_INVALID, "the deck does not use Stork tracking");
  th_status st = th_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (st != TH_OK) return st;
  const RunState* r = ctx->run;
  const int64_t n = r ? r->rows : 0;
  if (rows) *rows = n;
  const int64_t m = std::min<int64_t>(std::max<int64_t>(cap, 0), n);
  if (m == 0) return TH_OK;
  if (idx && (st = th_cuda_check(ctx, cudaMemcpy(idx, r->r_idx, 3 * m * sizeof(uint32_t), cudaMemcpyDeviceToHost),
                                 "cudaMemcpy")) != TH_OK)
    return st;
  if (ts && (st = th_cuda_check(ctx, cudaMemcpy(ts, r->r_ts, 2 * m * sizeof(double), cudaMemcpyDeviceToHost),
                                "cudaMemcpy")) != TH_OK)
    return st;
  if (Ts && (st = th_cuda_check(ctx, cudaMemcpy(Ts, r->r_Ts, 16 * m * sizeof(double), cudaMemcpyDeviceToHost),
                                "cudaMemcpy")) != TH_OK)
    return st;
  return TH_OK;
}

th_status th_output_rrdf(th_ctx* ctx, const char* name, int32_t binary) {
  if (!ctx || !name) return th_fail(ctx, TH_ERR_INVALID, "null argument");
  int64_t n = 0;
  th_status st = th_rrdf(ctx, nullptr, nullptr, nullptr, 0, &n);
  if (st != TH_OK) return st;
  std::vector<uint32_t> idx(3 * (size_t)n);
  std::vector<double> ts(2 * (size_t)n), Ts(16 * (size_t)n);
  int64_t got = 0;
  if ((st = th_rrdf(ctx, idx.data(), ts.data(), Ts.data(), n, &got)) != TH_OK) return st;
  std::string err;
  const bool ok = binary ? th_write_rrdf_bin(ctx->hp, name, idx.data(), ts.data(), Ts.data(), n, err)
                         : th_write_rrdf_csv(ctx->hp, name, idx.data(), ts.data(), Ts.data(), n, err);
  return ok ? TH_OK : th_fail(ctx, TH_ERR_IO, err);
}

th_status th_rdf(th_ctx* ctx, int32_t* counts, double* vals, int64_t cap, int64_t* nvals) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  if (!ctx->hp.o_rdf) return th_fail(ctx, TH_ERR_INVALID, "the deck does not ask for RDF output");
  if (!ctx->run) return th_fail(ctx, TH_ERR_INVALID, "run th_solidify first");
  th_status st = th_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (st != TH_OK) return st;
  RdfHost h;
  if ((st = gather_rdf(ctx, h)) != TH_OK) return st;
  const int64_t n = (int64_t)(h.tm.size() + 2 * h.sol.size());
  if (nvals) *nvals = n;
  if (counts) {
    std::fill(counts, counts + 3 * ctx->hp.pnum, 0);
    for (const auto& e : h.tm) counts[3 * (int64_t)e.first] += 1;
    for (const RdfSol& e : h.sol) { counts[3 * (int64_t)e.p + 1] += 1; counts[3 * (int64_t)e.p + 2] += 1; }
  }
  if (vals) {
    int64_t o = 0;
    size_t a = 0, b = 0;
    while ((a < h.tm.size() || b < h.sol.size()) && o < cap) {
      const int p = std::min(a < h.tm.size() ? h.tm[a].first : INT_MAX, b < h.sol.size() ? h.sol[b].p : INT_MAX);
      size_t a1 = a, b1 = b;
      while (a1 < h.tm.size() && h.tm[a1].first == p) ++a1;
      while (b1 < h.sol.size() && h.sol[b1].p == p) ++b1;
      for (size_t i = a; i < a1 && o < cap; ++i) vals[o++] = h.tm[i].second;
      for (size_t i = b; i < b1 && o < cap; ++i) vals[o++] = h.sol[i].tsol;
      for (size_t i = b; i < b1 && o < cap; ++i) vals[o++] = h.sol[i].cr;
      a = a1; b = b1;
    }
  }
  return TH_OK;
}

// <name>T.hist.csv of a deck with Output T_hist 1 (bin/Main.cpp:113-115).
static th_status write_T_hist(th_ctx* ctx) {
  if (!ctx->hp.o_T_hist) return TH_OK;
  std::string err;
  if (!th_write_T_hist_csv(ctx->hp, "T.hist", ctx->hist_t.data(), ctx->hist_T.data(), (int64_t)ctx->hist_t.size(), err))
    return th_fail(ctx, TH_ERR_IO, err);
  return TH_OK;
}

th_status th_T_hist(th_ctx* ctx, double* times, double* T, int64_t cap, int64_t* ntimes) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  if (!ctx->hp.o_T_hist) return th_fail(ctx, TH_ERR_INVALID, "the deck does not ask for T_hist output");
  const int64_t n = (int64_t)ctx->hist_t.size();
  if (ntimes) *ntimes = n;
  const int64_t m = std::min<int64_t>(std::max<int64_t>(cap, 0), n);
  if (times) std::copy(ctx->hist_t.begin(), ctx->hist_t.begin() + m, times);
  if (T) std::copy(ctx->hist_T.begin(), ctx->hist_T.begin() + m * ctx->hp.pnum, T);
  return TH_OK;
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
    ctx->hist_t.clear();
    ctx->hist_T.clear();
    for (int i = 0; i < (int)hp.snaps.size(); ++i) {
      th_status st = th_snapshot(ctx, i, T.data());
      if (st != TH_OK) return st;
      std::string err;
      if (!th_write_csv(hp, "Snapshot." + th_zero_pad(i, 2), names, cols, nullptr, err))
        return th_fail(ctx, TH_ERR_IO, err);
      if (hp.o_T_hist) {                      // each snapshot's T joins the history (src/Run.cpp:109)
        try {
          ctx->hist_t.push_back(hp.snaps[i]);
          ctx->hist_T.insert(ctx->hist_T.end(), T.begin(), T.end());
        } catch (const std::bad_alloc&) {
          return th_fail(ctx, TH_ERR_CAPACITY, "the T_hist history does not fit in host memory");
        }
      }
    }
    return write_T_hist(ctx);
  }
  th_status st = th_cuda_check(ctx, cudaSetDevice(ctx->device), "cudaSetDevice");
  if (st != TH_OK) return st;
  if (!ctx->run && (st = init_run(ctx)) != TH_OK) return st;
  if (hp.tracking == TH_TRACK_STORK) {
    // Stork writes its doubly reduced data in place of Solidification.Final and no
    // intermediate files (bin/Main.cpp:104-111, src/Run.cpp:711-1079)
    while (!ctx->run->done)
      if ((st = advance(ctx, (int64_t)INT_MAX - 1)) != TH_OK) return st;
    if ((st = th_output_rrdf(ctx, "RRDF", 0)) != TH_OK) return st;
    return hp.o_rdf ? write_rdf_csv(ctx, "RDF.Final") : TH_OK;
  }
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
  if ((st = write_solidification_csv(ctx, "Solidification.Final")) != TH_OK) return st;
  // the temperature history, then the reduced data, after the grid's fields (bin/Main.cpp:104-119)
  if ((st = write_T_hist(ctx)) != TH_OK) return st;
  return hp.o_rdf ? write_rdf_csv(ctx, "RDF.Final") : TH_OK;
}

}  // extern "C"
