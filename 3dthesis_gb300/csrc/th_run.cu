// Mode drivers behind th_simulate / th_solidify / th_field.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "th_ctx.h"
#include "th_output.h"

struct RunState {};

void th_release_run_state(th_ctx* ctx) {
  delete ctx->run;
  ctx->run = nullptr;
}

extern "C" {

th_status th_solidify(th_ctx* ctx, int64_t max_steps, int64_t* steps_out) {
  (void)max_steps; (void)steps_out;
  return th_fail(ctx, TH_ERR_UNSUPPORTED, "solidification is not built yet");
}

th_status th_field(th_ctx* ctx, const char* name, double* out) {
  if (!ctx || !name || !out) return th_fail(ctx, TH_ERR_INVALID, "null argument");
  cudaSetDevice(ctx->device);
  const std::string f(name);
  const int64_t n = ctx->hp.pnum;
  if (f == "T") {
    if (!ctx->T_valid) return th_fail(ctx, TH_ERR_INVALID, "no temperature field computed yet");
    cudaError_t e = cudaMemcpy(out, ctx->d_T, n * sizeof(double), cudaMemcpyDeviceToHost);
    return th_cuda_check(ctx, e, "cudaMemcpy");
  }
  if (f == "output_flag" && ctx->hp.mode == 0) {
    for (int64_t p = 0; p < n; ++p) out[p] = 1.0;
    return TH_OK;
  }
  return th_fail(ctx, TH_ERR_INVALID, "field " + f + " is not available");
}

th_status th_simulate(th_ctx* ctx) {
  if (!ctx) return th_fail(ctx, TH_ERR_INVALID, "null context");
  const HostProblem& hp = ctx->hp;
  if (hp.mode != 0) return th_solidify(ctx, 0, nullptr);
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

}  // extern "C"
