/*
 * TEST INFRASTRUCTURE ONLY.  CPU restatement of the 3DThesis hot path, used as the
 * parity oracle and as the timed CPU baseline.  Nothing in the product links it.
 *
 * It restates, in double precision and in the reference's own operation order:
 *   - the keyword-file input layer            (src/Init.cpp:33-908)
 *   - quadrature-node generation              (src/Calc.cpp:48-211, src/Util.cpp:40-50,145-237)
 *   - method-of-images boundary nodes         (src/Calc.cpp:503-608)
 *   - the point x node temperature sum        (src/Grid.cpp:275-314)
 *   - solidification time / G / V / dT/dt     (src/Grid.cpp:316-453, 522-548)
 *   - beam trace, frontier expansion, depth   (src/Melt.cpp:20-357)
 *   - the snapshot and solidification drivers (src/Run.cpp:80-124, 409-709)
 *
 * Pinned against the reference itself: tests/golden/ holds vectors produced by the
 * reference compiled from its own sources (oracle/Makefile, target "ref").
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parse a deck (ParamInput.txt).  Returns an opaque handle or NULL (message in err). */
void* or_load(const char* param_input, char* err, int errlen);
void  or_free(void* h);

/* info[0..15]: nx, ny, nz, pnum, n_beams, n_snapshots, mode(0 snap,1 sol),
 * tracking(0 None,1 Volume,2 Surface), dt, end_time, T0, TL, r_max, a, threads, use_bcs */
void  or_info(void* h, double* info);
double or_snapshot_time(void* h, int idx);

/* Quadrature nodes at t (reference field order: xb yb zb 1/phix 1/phiy 1/phiz dtau expmod),
 * written as 8 consecutive arrays of length cap.  Returns the node count (may exceed cap:
 * then only cap are written). */
int   or_nodes(void* h, double t, int is_sol, double* out, int cap);

/* T at the given points (flat ids, k fastest) from the nodes at t.  threads<=0: all. */
void  or_calc_T(void* h, double t, const int64_t* pts, int64_t n, double* T, int threads);

/* Snapshot idx over the whole grid (Snapshots_NoTracking). */
void  or_snapshot(void* h, int idx, double* T, int threads);

/* Full solidification run (Solidify_NoTracking / _Volume / _Surface).  max_steps<=0: until
 * the reference's finish test.  Returns the number of steps run. */
int64_t or_solidify(void* h, int threads, int64_t max_steps);

/* The same, also stopping after the first step that ends more than budget_s seconds of wall
 * time after the start (budget_s <= 0: no limit); for timing a bounded prefix of a run. */
int64_t or_solidify_budget(void* h, int threads, int64_t max_steps, double budget_s);

/* Per-point field after or_solidify: "T", "tSol", "G", "V", "Gx", "Gy", "Gz", "dTdt",
 * "eqFrac", "numMelt", "depth", "output_flag"; and for the tests' explanations "band" (the
 * closest approach of an evaluated T to T_L, DBL_MAX if never evaluated) and "sol_dT" (T -
 * T_last of the latest solidification's secant, 0 if none).  Returns 0 on success. */
int   or_field(void* h, const char* name, double* out);

/* G, Gx/G, Gy/G, Gz/G, dT/dt, V, eqFrac of point p for a solidification time tsol
 * (the second half of Grid::Solidify), into out[0..6]; then the cooling rate before its
 * integer truncation, the magnitude of its terms and the magnitude of the gradient's terms
 * (out[7..9]: how well the fields are conditioned). */
void  or_solid_fields(void* h, int64_t p, double tsol, double* out);
/* The same for n points, out[10 * i ...]. */
void  or_solid_fields_many(void* h, const int64_t* pts, const double* tsol, int64_t n, double* out, int threads);

/* Signature (64-bit hash) of the discrete choices of the quadrature walk at t: segments,
 * interval cuts, step-cap doublings, Gauss orders and kept nodes.  Equal signatures at two
 * times mean the node lists are the same continuous function of t between them. */
uint64_t or_schedule(void* h, double t, int is_sol);
void  or_schedule_many(void* h, const double* t, int64_t n, int is_sol, uint64_t* out, int threads);

/* After a run with Output RDF 1: per point (in point order) the numbers of melting times,
 * solidification times and cooling rates (counts[3p .. 3p+2]), and all values in that order
 * (per point its melting times, then solidification times, then cooling rates); dT gets
 * per solidification time its secant's T - T_last.  Returns the number of values (-1
 * without RDF); copies at most cap into each array. */
int64_t or_rdf(void* h, int32_t* counts, double* vals, double* dT, int64_t cap);

/* After a Stork run (Tracking Stork): the doubly reduced data, rows in the reference's
 * single-thread order (step, then cell): per row the cell index (3), the two step times (2)
 * and the 16 vertex temperatures.  Returns the row count; copies at most cap rows. */
int64_t or_rrdf(void* h, uint32_t* idx, double* ts, double* Ts, int64_t cap);

/* Point x node pairs evaluated since load (temperature sums + gradient sums). */
int64_t or_pairs(void* h);

#ifdef __cplusplus
}
#endif
