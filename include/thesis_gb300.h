/*
 * thesis_gb300 - C ABI of the GB300 (sm_103a) implementation of the 3DThesis hot path:
 * the time integral of the moving 3D-Gaussian heat source, summed over adaptive Gauss
 * quadrature nodes on the scan path, at every tracked grid point.
 *
 * Plain C types only (no CUDA or torch types).  Every call returns a th_status; on an
 * error th_last_error(ctx) (or th_last_error(NULL) for failed creation) describes it.
 * A context owns every device buffer it uses and is bound to the CUDA device that was
 * current when it was created.  Contexts are independent; one context must not be used
 * from two host threads at once.
 *
 * Reference interfaces each entry point replaces (paths inside the 3DThesis tree):
 *   th_ctx_create_from_deck  Init::GetFileNames + Init::ReadSimParams + Grid(sim)
 *                            (src/Init.cpp:233-303, src/Grid.h:120-280, bin/Main.cpp:62-74)
 *   th_nodes                 Calc::Integrate_Serial (src/Calc.h:23, src/Calc.cpp:48-65)
 *   th_calc_T                Grid::Calc_T with set = false over many points
 *                            (src/Grid.h:290, src/Grid.cpp:275-314)
 *   th_snapshot              one iteration of Run::Snapshots_NoTracking (src/Run.cpp:80-124)
 *   th_solidify              Run::Solidify (src/Run.cpp:390-709): NoTracking, Volume, Surface
 *   th_simulate              Run::Simulate + the final outputs of bin/Main.cpp:88-118
 *   th_field                 the Grid getters (src/Grid.h:299-370)
 */
#ifndef THESIS_GB300_H
#define THESIS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int th_status;
enum {
  TH_OK = 0,
  TH_ERR_INVALID = 1,      /* bad argument or input deck */
  TH_ERR_IO = 2,           /* file could not be read or written */
  TH_ERR_CUDA = 3,         /* a CUDA call failed */
  TH_ERR_CAPACITY = 4,     /* a fixed-size buffer or limit was exceeded */
  TH_ERR_UNSUPPORTED = 5,  /* a reference feature this build does not implement */
  TH_ERR_TIMEOUT = 6       /* a bounded device loop gave up */
};

/* Arithmetic of the point x node sums. */
enum {
  TH_FP64 = 0,        /* plain double precision, the reference's arithmetic */
  TH_FP32_KAHAN = 1   /* FP32 pair terms, Kahan-compensated FP32 sums, FP64 node
                         generation and FP64 node-to-tile offsets */
};

typedef struct th_ctx th_ctx;

typedef struct th_info {
  int32_t nx, ny, nz;          /* grid points per axis (k fastest: p = i*ny*nz + j*nz + k) */
  int64_t pnum;                /* nx*ny*nz */
  int32_t n_beams;
  int32_t n_snapshots;
  int32_t mode;                /* 0 Snapshots, 1 Solidification */
  int32_t tracking;            /* 0 None, 1 Volume, 2 Surface, 3 Stork */
  double dt;                   /* solidification timestep (s) */
  double end_time;             /* end of the last scan path (s) */
  double T0, TL;               /* initial and liquidus temperature (K) */
  double xmin, xmax, ymin, ymax, zmin, zmax;
  int32_t precision;
  int32_t out_flags;           /* bit mask of requested output fields, TH_OUT_* */
} th_info;

/* Output field bits (the reference's Output.txt keywords). */
enum {
  TH_OUT_T = 1 << 0, TH_OUT_TSOL = 1 << 1, TH_OUT_G = 1 << 2, TH_OUT_GX = 1 << 3,
  TH_OUT_GY = 1 << 4, TH_OUT_GZ = 1 << 5, TH_OUT_V = 1 << 6, TH_OUT_DTDT = 1 << 7,
  TH_OUT_EQFRAC = 1 << 8, TH_OUT_DEPTH = 1 << 9, TH_OUT_NUMMELT = 1 << 10
};

/* Creates a context from a deck's ParamInput.txt.  File names inside the deck are
 * resolved relative to the directory of param_input (the reference opens them relative
 * to its working directory, which is that directory when run as `3DThesis ParamInput.txt`). */
th_status th_ctx_create_from_deck(const char* param_input, int32_t precision, th_ctx** out);
void th_ctx_destroy(th_ctx* ctx);
const char* th_last_error(const th_ctx* ctx);
th_status th_get_info(th_ctx* ctx, th_info* out);
/* The same summary of a deck without a context or a GPU (host parsing only, as
 * Init::ReadSimParams does, src/Init.cpp:33-908): what a launcher needs to split work
 * across GPUs before any device is touched.  precision is reported as -1; errors go to
 * th_last_error(NULL). */
th_status th_deck_info(const char* param_input, th_info* out);
double th_snapshot_time(th_ctx* ctx, int32_t idx);

/* Quadrature nodes at time t (is_sol != 0: the refined solidification schedule).
 * Writes 8 arrays of length cap, in this order: xb, yb, zb, 1/phix, 1/phiy, 1/phiz, dtau,
 * expmod (the reference's Nodes fields).  *n_out receives the node count; when it exceeds
 * cap only the first cap nodes are written. */
th_status th_nodes(th_ctx* ctx, double t, int32_t is_sol, double* out, int32_t cap, int32_t* n_out);

/* T at n grid points (flat ids) from the nodes at t; host buffers.  pts == NULL means
 * every grid point (n must then equal pnum). */
th_status th_calc_T(th_ctx* ctx, double t, const int64_t* pts, int64_t n, double* T_out);

/* The same with device buffers, enqueued on `stream` (a cudaStream_t; NULL = the
 * context's own stream).  Returns after enqueueing, without synchronising: a device-side
 * failure (node list larger than its buffer, walk step limit) is reported by th_sync or by
 * the next synchronous call on the context. */
th_status th_calc_T_device(th_ctx* ctx, double t, const int64_t* d_pts, int64_t n, double* d_T,
                           void* stream);

/* Allocation-free form of th_calc_T_device, for callers that cannot allocate device
 * memory or let the library allocate it (their device memory is owned by their own pool
 * or a budget fixed at start-up, or the call sits in a time loop where cudaMalloc /
 * cudaFree would synchronise the device and could fail).  No counterpart in the reference.
 * It calls no cudaMalloc, cudaFree or other allocating routine: the node list lives in a
 * static device array of the library holding at most 16384 nodes (about 1.7 MB, kept by
 * every GPU that loads the library until the process exits); a longer list returns
 * TH_ERR_CAPACITY and leaves d_T invalid.  The first call on a device looks the array's
 * address up once for that device.  It synchronises `stream` before returning (to report
 * that error).  Every call, from every context on the device, shares the one array, so
 * calls that overlap on the GPU (other streams or host threads) race and must be
 * serialised by the caller. */
th_status th_calc_T_noalloc(th_ctx* ctx, double t, const int64_t* d_pts, int64_t n, double* d_T,
                            void* stream);

/* Waits for `stream` (NULL: only the context's own stream) and reports any device-side
 * error latched since the last check. */
th_status th_sync(th_ctx* ctx, void* stream);

/* T at ntimes times into d_T + i * n (device memory): the node lists of all times in one
 * launch, one block per time (Calc::Integrate_Parallel, src/Calc.cpp:21-46, precomputes
 * future lists the same way), then one sum per time.  Same stream semantics and latched
 * errors as th_calc_T_device; successive calls must use one stream. */
th_status th_calc_T_times_device(th_ctx* ctx, const double* times, int32_t ntimes, const int64_t* d_pts, int64_t n,
                                 double* d_T, void* stream);

/* Snapshot idx of a Snapshots deck over the whole grid: T for every point (host buffer,
 * pnum doubles).  T_out == NULL leaves the result in the context's device buffer. */
th_status th_snapshot(th_ctx* ctx, int32_t idx, double* T_out);

/* Runs the Solidification loop of the deck on the device.  max_steps <= 0 runs to the
 * reference's finish test (t past the end of every path and no liquid point left).
 * *steps_out (may be NULL) receives the number of timesteps taken. */
th_status th_solidify(th_ctx* ctx, int64_t max_steps, int64_t* steps_out);

/* Copies a per-point field (pnum doubles) to host memory after th_snapshot/th_solidify:
 * "T", "tSol", "G", "V", "Gx", "Gy", "Gz", "dTdt", "eqFrac", "numMelt", "depth",
 * "output_flag". */
th_status th_field(th_ctx* ctx, const char* name, double* out);

/* Discards the solidification state (the next th_solidify starts again at t = 0). */
th_status th_run_reset(th_ctx* ctx);

/* Device time and counters of the solidification loop so far, out[0..n): ms building
 * node windows, ms in the tracking / NoTracking steps, ms solidifying records, windows,
 * records, most work items in one step (tracking), steps, node slots per step,
 * device-elapsed ms of th_solidify calls (host gaps included), point x node pairs of the
 * bulk solidification, all point x node pairs of the context; then the tracking loop's
 * profile: ms of block 0's work phases, 0 (a slot kept for a barrier time; the loop has
 * no grid barrier), work items run,
 * SM clocks spent in items and in waiting for items (summed over warps), the per-step
 * longest parent -> child item chain summed over steps, steps profiled, point evaluations
 * and their SM clocks summed over warps, then per chain depth 0, 1, 2, >= 3 the latest
 * item start and the latest item end after the step began, in ms summed over steps, the
 * nodes of the evaluation passes summed over passes, the records of an FP32 run whose
 * solidification was redone in FP64, the liquid decisions of an FP32 run taken on an
 * FP64 sum, for Stork tracking the ms building the doubly reduced data and its rows, and
 * the records of an FP32 run re-solidified from FP64 temperatures (34 values). */
th_status th_run_stats(th_ctx* ctx, double* out, int32_t n);

/* After th_solidify / th_simulate of a deck with Output RDF 1: the reduced data of the run
 * so far as the reference's Grid holds it (Grid::get_RDF_tm / _tl / _cr,
 * src/Grid.h:360-362): counts gets per point (3 * pnum values) its numbers of melting
 * times, solidification times and cooling rates; vals gets, point by point in point order,
 * its melting times, then solidification times, then cooling rates, each in time order (at
 * most cap values); *nvals receives the number of values.  Melting times are kept by
 * Surface tracking only (src/Run.cpp:604-609), as in the reference.  Either array may be
 * null. */
th_status th_rdf(th_ctx* ctx, int32_t* counts, double* vals, int64_t cap, int64_t* nvals);

/* After th_solidify / th_simulate of a Stork deck (Tracking Stork): the doubly reduced data
 * of the run so far, the rows in step order and within a step in ascending cell index
 * (the reference's single-thread order).  Per row: idx the cell's (i, j, k) (3 values),
 * ts the previous and the current step time (2), Ts the temperatures of the cell's 8
 * vertices at the previous step, then at the current one, vertex (di, dj, dk) at
 * di*4 + dj*2 + dk (16).  Copies min(cap, rows) rows into each non-null array; *rows
 * receives the row count.  Replaces Grid::get_RRDF_idxs / get_RRDF_ts / get_RRDF_Ts
 * (src/Grid.h:368-370), filled by Run::Stork (src/Run.cpp:711-1079). */
th_status th_rrdf(th_ctx* ctx, uint32_t* idx, double* ts, double* Ts, int64_t cap, int64_t* rows);

/* The same rows as a file: <deck dir>/Data/<deck name>.<name>.csv (binary 0, the columns of
 * th_simulate's RRDF file) or .bin (binary 1: the row count as uint32, the grid's point
 * counts as 3 x uint32, its x, y, z minima, x resolution and the liquidus as 5 x double,
 * then every row's 3 indices as uint32, 2 times and 16 temperatures as double, block by
 * block, in the machine's byte order).  Replaces Grid::Output_RRDF_csv / Output_RRDF_bin
 * (src/Grid.cpp:203-273).  TH_ERR_IO if the file cannot be written. */
th_status th_output_rrdf(th_ctx* ctx, const char* name, int32_t binary);

/* With Output T_hist 1 (Tracking None only: every point is evaluated at the same times):
 * the temperature history th_simulate or th_solidify collected - times the evaluation times
 * (Snapshots: the snapshot times; Solidification: every step the loop ran), T time by time
 * every point's temperature (pnum values per time, in point order).  Copies min(cap,
 * ntimes) times and their rows into each non-null array; *ntimes receives the count.
 * Replaces Grid::get_t_hist / get_T_hist (src/Grid.h:357-358), filled by Grid::Calc_T with
 * set (src/Grid.cpp:300-304); th_simulate writes them as <name>T.hist.csv
 * (Grid::Output_T_hist, src/Grid.cpp:101-136). */
th_status th_T_hist(th_ctx* ctx, double* times, double* T, int64_t cap, int64_t* ntimes);

/* Whole run as the reference CLI does it: the mode loop, then the CSV files under
 * <deck dir>/Data (same names, columns and number format; a Stork deck writes
 * <name>.RRDF.csv in place of <name>.Solidification.Final.csv; Output RDF 1 adds
 * <name>.RDF.Final.csv; Output T_hist 1 adds <name>T.hist.csv). */
th_status th_simulate(th_ctx* ctx);

/* Point x node pairs evaluated by this context so far (temperature and gradient sums). */
th_status th_pairs(th_ctx* ctx, int64_t* out);

/* Tile shape of the whole-grid kernels: kp k-points per thread, kch k-chunks per tile
 * (supported: kp 4 with kch 1/2/4, kp 2 with kch 2/4, kp 8 with kch 1/2). */
th_status th_set_tile_shape(th_ctx* ctx, int32_t kp, int32_t kch);

/* Device time (ms) of the most recent th_snapshot's point x node kernel. */
th_status th_last_kernel_ms(th_ctx* ctx, float* out);

/* Issue rates of the current device, measured with throughput-bound probe kernels, for
 * the roofline the point x node kernels are measured against.  No counterpart in the
 * reference (it has no GPU code).  out[0] SM count, out[1] the device's maximum SM clock
 * (MHz), out[2] MUFU ex2 results per SM per clock, out[3] FP32 FMA lane-operations per SM
 * per clock. */
th_status th_device_rates(double* out);

/* Times snapshot idx's whole-grid kernel with every supported tile shape and keeps the
 * fastest for this context; the chosen shape is written to *kp_out / *kch_out. */
th_status th_autotune(th_ctx* ctx, int32_t idx, int32_t* kp_out, int32_t* kch_out);

/* ---- Batched snapshots -------------------------------------------------------------
 * n independent Snapshots decks (a process-parameter sweep: power, speed, widths,
 * material, path, grid may all differ) evaluated together.  A batch snapshot fills one
 * flat array: deck d's grid occupies [offsets[d], offsets[d + 1]) in the deck's own point
 * order.  Snapshot idx of the batch is snapshot idx of every deck (idx below the smallest
 * snapshot count).  Each batch snapshot is two launches - node lists, one thread block per
 * deck, and a persistent work-list kernel over every deck's tiles - captured once as a CUDA
 * graph and replayed.  The reference runs such sweeps as one process per deck
 * (bin/Main.cpp:45-94 runs one ParamInput.txt per process). */
typedef struct th_batch th_batch;

th_status th_batch_create(const char* const* param_inputs, int32_t n, int32_t precision, th_batch** out);
void th_batch_destroy(th_batch* b);
/* Message of the last failure on b (b NULL: of the last failed th_batch_create). */
const char* th_batch_last_error(const th_batch* b);
/* offsets[0..n]: exclusive prefix of the decks' point counts. */
th_status th_batch_points(th_batch* b, int64_t* offsets);
/* Snapshot idx of every deck into host memory T_out (offsets[n] doubles); synchronous. */
th_status th_batch_snapshot(th_batch* b, int32_t idx, double* T_out);
/* The same into device memory d_T, enqueued on stream (NULL: the batch's own stream);
 * returns without waiting.  Node-list errors surface at the next th_batch_snapshot. */
th_status th_batch_snapshot_device(th_batch* b, int32_t idx, double* d_T, void* stream);
th_status th_batch_set_tile_shape(th_batch* b, int32_t kp, int32_t kch);
/* Times every supported tile shape on batch snapshot idx and keeps the fastest. */
th_status th_batch_autotune(th_batch* b, int32_t idx, int32_t* kp_out, int32_t* kch_out);
/* Point x node pairs evaluated by the batch so far. */
th_status th_batch_pairs(th_batch* b, int64_t* out);

/* ---- Adjoint (calibration gradients) -----------------------------------------------
 * Temperatures of a single-beam deck at probe points and times, as a function of the
 * parameter vector theta = (P, efficiency, Width_X, Width_Y, Depth_Z, alpha, then x, y of
 * every path vertex after the origin, in metres), and the gradient of a loss through them.
 * alpha is the diffusivity k / (rho c).  The node list is re-walked for theta on the host in
 * FP64 dual numbers (values identical to the device walk); the device recomputes each
 * probe x node term for the per-node adjoint sums.  The walk's discrete choices (interval
 * counts, Gauss orders, r_max cut-off) are held at theta's.  No reference counterpart: the
 * reference has no gradients (its forward is src/Calc.cpp:67-211 + src/Grid.cpp:275-314). */
typedef struct th_adj th_adj;

/* probes: flat grid point ids (k fastest); times: seconds.  No device work until forward. */
th_status th_adj_create(const char* param_input, int32_t precision, const int64_t* probes, int32_t nprobe,
                        const double* times, int32_t ntimes, th_adj** out);
void th_adj_destroy(th_adj* a);
const char* th_adj_last_error(const th_adj* a);
/* 6 + 2 x (path segments after the origin). */
int32_t th_adj_num_params(const th_adj* a);
/* The deck's own parameter values. */
th_status th_adj_params(th_adj* a, double* theta);
/* Host node list at times[time_idx] for theta (8 arrays of cap: x y z 1/phix 1/phiy 1/phiz
 * dtau amp) and, when tangents is not NULL, d(node field)/d(theta) laid out
 * [field][node][param] with cap nodes per field; *n_out = node count.  CPU only. */
th_status th_adj_host_nodes(th_adj* a, const double* theta, int32_t time_idx, double* out, int32_t cap,
                            double* tangents, int32_t* n_out);
/* T at every probe and time for theta: T_out[t * nprobe + p].  Remembers theta. */
th_status th_adj_forward(th_adj* a, const double* theta, double* T_out);
/* dL/dtheta from dL/dT (same layout as T_out) at the theta of the last forward. */
th_status th_adj_backward(th_adj* a, const double* dL_dT, double* dL_dtheta);

#ifdef __cplusplus
}
#endif
#endif /* THESIS_GB300_H */
