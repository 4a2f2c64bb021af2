// Solidification-mode device state and kernels (NoTracking, Volume, Surface).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "th_kernels.h"
#include "th_problem.h"

// One liquid -> solid transition seen by the tracking loop; the solidification time and
// the gradients are computed later, in bulk, from these four numbers
// (the inputs of Grid::Solidify, src/Grid.cpp:316-338).
struct SolRec {
  int32_t p;       // point id
  int32_t step;    // timestep index
  double t;        // time of the step
  double T;        // temperature at t
  double Tl;       // temperature at the previous step (T_last)
};

// Per-step counters; one struct in device memory.  Lists rotate over three buffers by
// step (k % 3: this step's liquid list, (k + 1) % 3: the next one, (k + 2) % 3: being
// cleared), so no buffer is reset while another block may still read it.
struct QueueCounters {
  unsigned head;                 // tickets taken
  unsigned unused;
  unsigned long long state;      // (dynamic items published << 32) | items completed; the
                                 // published count also hands out the items' queue slots
  unsigned pad[4];
};

struct TrackCounters {
  int liq_n[3];     // liquid list lengths
  int rec_n[2];     // solidification records queued in each of the two record buffers
  int step;         // next step to run
  int done;         // finish test passed
  int stop;         // the loop stopped early (record queue high-water mark)
  int max_items;    // most work items in one step
  int diag[8];      // where a bounded wait gave up: kind, step, ticket, n_init, head, tail, published, completed
  QueueCounters q[3];
};

// Device pointers of the solidification state.
struct TrackState {
  double* T;
  double* T_last;          // NoTracking only
  unsigned* stamp;         // claim stamp: claimed in step k <=> stamp >= k + 1
  unsigned char* outflag;  // output_flag
  int* last_liq;           // last step at which the point was liquid (-1: never)
  int* num_melt;
  int* sol_step;           // step of the record whose results are stored (-1: none)
  double* tSol; double* G; double* V; double* Gx; double* Gy; double* Gz; double* dTdt; double* eqFrac;
  double* depth;           // per point (Surface with depth output), may be null
  int* depths;             // per (i, j) column: deepest liquid layer
  double* depth_max;       // per column
  int* liq[3];
  int list_cap;
  int4* queue;             // work items {tag, type, point, aux}
  int queue_cap;
  SolRec* rec;             // the record buffer this launch appends to
  int* rec_n;              // and its length (one of TrackCounters::rec_n)
  int rec_cap;
  TrackCounters* C;
  unsigned* bar;           // grid barrier: [0] arrivals, [1] generation
  int* err;
  unsigned long long* pairs;
};

// A window of precomputed node lists: slot s holds the list of step (base - 1 + s).
struct NodeWindow {
  NodeBufView nb;          // slot-major: slot s starts at s * slot_cap
  int slot_cap;
  int nslots;
  int* count;              // per slot
  const double* t;         // per slot
  int base;                // step of slot 1
};

// Error bits written by the solidification kernels (besides the node bits).
enum { ERR_BARRIER = 16, ERR_RECORDS = 32, ERR_LISTS = 64, ERR_QUEUE = 128 };

void th_launch_nodes_window(const DevProblem& P, const NodeWindow& w, int first_slot, int nslots, bool is_sol,
                            int* d_err, cudaStream_t s);

// Runs steps [k_begin, k_end) of a Volume/Surface loop inside one cooperative launch.
cudaError_t th_launch_track(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k_begin, int k_end,
                            int precision, int rec_high_water, cudaStream_t s);

// One NoTracking step over the whole grid (src/Run.cpp:423-444).
void th_launch_notrack_step(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k, int precision,
                            cudaStream_t s);

// Solidification time, gradients and derived fields for nrec records of `rec`.
void th_launch_solidify(const DevProblem& P, const TrackState& S, const SolRec* rec, int nrec, int precision,
                        bool do_sol, cudaStream_t s);

// Final per-point field with the reference's liquid markers applied.
void th_launch_final_field(const DevProblem& P, const TrackState& S, int field, double* out, cudaStream_t s);

int th_track_blocks(int precision);
