// The context behind the C ABI's opaque th_ctx handle.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/thesis_gb300.h"
#include "th_kernels.h"
#include "th_problem.h"

struct RunState;   // solidification state (th_run.cu)

struct th_ctx {
  HostProblem hp;
  DevProblem dp;
  int precision = TH_FP32_KAHAN;
  int device = -1;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  std::string err;

  DevSeg* d_segs = nullptr;
  double* d_custom = nullptr;             // custom points' x, y, z (pnum each), null for a grid
  void* node_mem = nullptr;
  NodeBufView nb{};
  int* d_small = nullptr;                 // [0] node count, [1] error bits, [2..] scratch
  unsigned long long* d_pairs = nullptr;  // point x node pairs evaluated
  int last_count = 0;
  TileShape shape{4, 2};

  double* d_T = nullptr;       size_t T_bytes = 0;   bool T_valid = false;
  int64_t* d_pts = nullptr;    size_t pts_bytes = 0;
  double* d_Tlist = nullptr;   size_t Tlist_bytes = 0;
  double* d_export = nullptr;  size_t export_bytes = 0;

  RunState* run = nullptr;

  // the temperature history (Output T_hist 1, Tracking None): the evaluation times and, time
  // by time, every point's temperature, collected by th_simulate (snapshots) or the
  // solidification loop
  std::vector<double> hist_t, hist_T;

  // several node lists at once (th_calc_T_times_device): slot-major buffers of nb.cap nodes
  void* multi_mem = nullptr;   int multi_slots = 0;   int multi_cap = 0;
  double* d_multi_t = nullptr; int* d_multi_count = nullptr;
};

th_status th_fail(th_ctx* ctx, th_status code, const std::string& msg);
th_status th_cuda_check(th_ctx* ctx, cudaError_t e, const char* what);
th_status th_gen_nodes_checked(th_ctx* ctx, double t, bool is_sol);
th_status th_ensure(th_ctx* ctx, void** ptr, size_t* cap_bytes, size_t need);
void th_release_run_state(th_ctx* ctx);
