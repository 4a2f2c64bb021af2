// Command-line driver: `thesis_gb300 ParamInput.txt [fp32|fp64]`, the GB300 counterpart of
// the reference's `3DThesis ParamInput.txt` (bin/Main.cpp:44-124): reads the same deck,
// runs the mode on the GPU and writes the same CSV files under <deck dir>/Data, printing
// the same three timers.
#include <chrono>
#include <cstdio>
#include <cstring>

#include "../../include/thesis_gb300.h"

int main(int argc, char** argv) {
  if (argc <= 1) {
    std::fprintf(stderr, "Input file argument required: thesis_gb300 ParamInput.txt [fp32|fp64]\n");
    return 1;
  }
  const int precision = (argc > 2 && std::strcmp(argv[2], "fp64") == 0) ? TH_FP64 : TH_FP32_KAHAN;
  using clk = std::chrono::high_resolution_clock;
  const auto t0 = clk::now();
  th_ctx* ctx = nullptr;
  if (th_ctx_create_from_deck(argv[1], precision, &ctx) != TH_OK) {
    std::fprintf(stderr, "Fatal Error: %s\n", th_last_error(nullptr));
    return 1;
  }
  const auto t1 = clk::now();
  std::printf("Initialization time (s): %g\n\n", std::chrono::duration<double>(t1 - t0).count());
  const th_status st = th_simulate(ctx);
  const auto t2 = clk::now();
  if (st != TH_OK) {
    std::fprintf(stderr, "Error: %s\n", th_last_error(ctx));
    th_ctx_destroy(ctx);
    return 2;
  }
  std::printf("Execution time (s): %g\n\n", std::chrono::duration<double>(t2 - t1).count());
  th_ctx_destroy(ctx);
  return 0;
}
