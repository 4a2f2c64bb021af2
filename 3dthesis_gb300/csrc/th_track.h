// Solidification-mode device state and kernels (NoTracking, Volume, Surface, Stork).
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

// RDF (Output RDF 1): one solidification of a Surface run - its record's point and step, the
// solidification time and the cooling rate (Grid::Solidify's add_RDF_tl / add_RDF_cr,
// src/Grid.cpp:322,547) - and one melt event: a point still liquid when step `step` ended
// (pushed at the start of the next step as t - dt, src/Run.cpp:604-609).
struct RdfSol {
  int32_t p, step;
  double tsol, cr;
};

// A record of an FP32 run whose solidification is redone in FP64 (see k_solidify): the
// record's index, and why (bit 0: the gradient or cooling-rate sum was ill-conditioned for
// FP32 terms; bit 1: the solidification time was too sensitive to FP32 temperatures).
struct RedoRec {
  int32_t i;
  int32_t why;
};

// Per-step counters; one struct in device memory.  Lists rotate over three buffers by
// step (k % 3: this step's liquid list, (k + 1) % 3: the next one, (k + 2) % 3: being
// cleared), so no buffer is reset while another block may still read it.
//
// The counters that every warp touches live on separate 128-byte lines: the ticket
// counter, the published/completed word, and the finished-step stamp that idle warps poll,
// so the polling never queues behind the atomics.
struct alignas(128) QueueCounters {
  unsigned head;                 // tickets taken
  unsigned depth;                // longest parent -> child chain of the step's items
  unsigned lvl_start[4];         // latest start / end (ns after the step began) of the items of
  unsigned lvl_end[4];           // chain depth 0, 1, 2, >= 3 (profile)
  unsigned init_head;             // Volume: initial items taken (dealt by this counter, not by warp)
  unsigned pad0[21];
  unsigned long long state;      // the step word: items completed and published, blocks
                                 // entered (Surface forms: also liquid points and a stop
                                 // request; the layouts are StepWord's in th_track.cu); the
                                 // published count also hands out the items' queue slots
  unsigned long long pad1[15];
};

struct alignas(128) TrackCounters {
  int step;         // next step to run
  int done;         // finish test passed
  int stop;         // the loop stopped early (record queue high-water mark)
  int max_items;    // most work items in one step
  int diag[8];      // where a bounded wait gave up: 1, step, ticket, n_init, tickets taken, blocks entered, published, completed
  // loop profile: [0] block 0's work-phase time (ns), [1] unused (0; the loop has no grid
  // barrier), [2] items run, [3], [4] item and wait time summed over warps (SM clocks),
  // [5] summed per-step chain depth, [6] steps profiled, [7], [8], [9] evaluation passes,
  // their SM clocks and their nodes summed over warps, [10..13], [14..17] the per-step
  // latest start and end of items of chain depth 0..3 (ns) summed over steps
  unsigned long long prof[18];
  unsigned long long redo_total;   // FP32 runs: records whose solidification was redone in FP64
  unsigned long long guard_total;  // FP32 runs: liquid decisions taken on an FP64 sum
  unsigned long long fix_total;    // FP32 runs: records re-solidified from FP64 temperatures
                                   // (the three read with prof as its 19th to 21st words)
  alignas(128) int liq_n[3];     // liquid list lengths
  alignas(128) int rec_n[2];     // solidification records queued in each of the two record buffers
  alignas(128) int tm_n[2];      // RDF melt events logged in each of the two event buffers
  // once step k is over: (next step's liquid-list length << 34) | (flags << 32) | (k + 1), flags
  // 1 finished run, 2 launch ends (a record buffer or log at its high-water mark); low word
  // 0xffffffff: aborted by a bounded wait
  alignas(128) unsigned long long fin;
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
  int2* liq[3];             // liquid surface points (point, column depth), rotating by step
  int list_cap;
  ulonglong2* queue;       // work items {stamp << 32 | point, stamp << 32 | type | depth << 8 | aux << 16}
  int queue_cap;
  SolRec* rec;             // the record buffer this launch appends to
  int* rec_n;              // and its length (one of TrackCounters::rec_n)
  int rec_cap;
  RedoRec* redo;           // FP32 runs: records queued for the FP64 redo of their solidification
  int* redo_n;             // (capacity rec_cap; emptied after each redo pass)
  RedoRec* fix;            // FP32 runs: records whose secant only needs FP64 temperatures, their
  int* fix_n;              // count, and those temperatures (T, T_last) (capacity rec_cap)
  double2* fix_T;
  NodeBufView redo_nb;     // FP32 runs: a scratch node list of redo_cap nodes per redo block
  int redo_cap;            // (block b's at b * redo_cap), and per block its list's count and
  int redo_blocks;         // error bits (redo_aux[2 b], redo_aux[2 b + 1])
  int* redo_aux;
  // RDF of Surface runs (null otherwise): per point the melt events opened minus the
  // solidifications (the reference's tm count minus its tl count: an event opens only at
  // 0), the launch's melt-event log (point, step) and its length, and the bulk
  // solidification's per-record results at rdf_base + record index
  int* rdf_open;
  int2* tm_log;
  int* tm_n;
  int tm_cap;
  RdfSol* rdf_sol;
  long long rdf_base;
  // Stork: the launch's log of liquid lists (entries as in liq: point, column depth); list j
  // (j = 0: the liquid points of step k_begin - 1, then one per step run) spans
  // [rlog_off[j], rlog_off[j + 1]); null for the other forms
  int2* rlog;
  int* rlog_off;
  int rlog_cap;
  int rlog_step_max;       // the longest list one step can add (a launch stops before the log
                           // has less room than that)
  TrackCounters* C;
  const float2* axis;      // grid coordinates as (hi, lo) floats: x[0, nx), y[nx, nx + ny), z after
  int t_fixed;             // T and the records' T, T_last hold FP32 tracking's fixed point (see t_decode)
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
  // beam-trace candidates of each slot's step (Volume / Surface tracking): surface points
  // the trace would test, before the claim; nseed[slot] may exceed seed_cap (overflow)
  int* seeds;              // slot-major, seed_cap per slot
  int* nseed;
  int seed_cap;
};

#ifdef __CUDACC__
// Slot `slot` of a window as a node-list view.
__device__ __forceinline__ NodeBufView slot_view(const NodeWindow& w, int slot) {
  NodeBufView v = w.nb;
  const size_t off = (size_t)slot * w.slot_cap;
  v.x += off; v.y += off; v.z += off; v.ipx += off; v.ipy += off; v.ipz += off; v.dtau += off; v.amp += off;
  v.kx += off; v.ky += off; v.kz += off; v.w += off; v.xh += off; v.xl += off; v.yh += off; v.yl += off;
  v.zh += off; v.zl += off;
  v.cap = w.slot_cap;
  return v;
}
#endif

// Error bits of a window build (with the node bits 1 = node capacity, 2 = walk limit).
enum { ERR_SEED_CAPACITY = 4 };

// Error bits written by the solidification kernels (besides the node bits).
enum { ERR_BARRIER = 16, ERR_RECORDS = 32, ERR_LISTS = 64, ERR_QUEUE = 128, ERR_RDF = 256 };

void th_launch_nodes_window(const DevProblem& P, const NodeWindow& w, int first_slot, int nslots, bool is_sol,
                            int* d_err, cudaStream_t s);

// Runs steps [k_begin, k_end) of a Volume/Surface loop inside one cooperative launch.
cudaError_t th_launch_track(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k_begin, int k_end,
                            int precision, int rec_high_water, cudaStream_t s);

// One NoTracking step over the whole grid (src/Run.cpp:423-444).
void th_launch_notrack_step(const DevProblem& P, const TrackState& S, const NodeWindow& w, int k, int precision,
                            cudaStream_t s);

// Solidification time, gradients and derived fields for nrec records of `rec`; `w` is the
// node window of the records' steps (the FP64 redo of FP32 runs reads the lists of each
// record's step and of the step before it).
void th_launch_solidify(const DevProblem& P, const TrackState& S, const NodeWindow& w, const SolRec* rec, int nrec,
                        int precision, bool do_sol, cudaStream_t s);

// Stork's doubly reduced data for the steps of one tracking launch (th_rrdf.cu): a count
// pass gives each step's rows and vertex values, then a fill pass writes the rows at the
// offsets the host lays out (cell index: 3 values, step times: 2, vertex temperatures: 16
// per row, as Grid::get_RRDF_idxs / _ts / _Ts hold them, src/Grid.h:368-370).
struct RrdfBatch {
  const int2* log;           // the launch's log of liquid lists (TrackState::rlog)
  const int* off;            // list j spans [off[j], off[j + 1]), j = 0 .. nsteps
  int k0, nsteps;            // step k0 + j has lists j (liquid at k - 1) and j + 1 (liquid at k)
  int nmax;                  // most entries of two consecutive lists
  int* counts;               // per step: rows, vertex values
  const long long* row_base; // fill: per step, its first row
  int* scratch;              // per block: th_rrdf_scratch_ints(nmax) ints
  double* vals;              // fill, per block: 3 * vals_cap doubles (vertex values, vertex ids)
  int vals_cap;
  uint32_t* idx;             // fill: the rows
  double* ts;
  double* Ts;
  int* err;                  // bit 0: a step had more vertex values than vals_cap
  unsigned long long* pairs; // the context's point x node pair count
};
size_t th_rrdf_scratch_ints(int nmax);
void th_launch_rrdf(const DevProblem& P, const NodeWindow& w, const RrdfBatch& b, bool fill, int precision, int blocks,
                    cudaStream_t s);

// Final per-point field with the reference's liquid markers applied.
void th_launch_final_field(const DevProblem& P, const TrackState& S, int field, double* out, cudaStream_t s);

int th_track_blocks(int precision);
