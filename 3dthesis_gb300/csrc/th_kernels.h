// Launch wrappers for the device kernels (host side).
#pragma once
#include <cuda_runtime.h>
#include "th_problem.h"

// Device node list: structure-of-arrays, capacity `cap`.
//  doubles: x y z ipx ipy ipz dtau amp   (amp = q beta / sqrt(phix phiy phiz))
//  floats : kx ky kz w                   (k = -3 log2(e) / phi, w = dtau * amp)
//           xh xl yh yl zh zl            (coordinates split into two floats)
struct NodeBufView {
  double *x, *y, *z, *ipx, *ipy, *ipz, *dtau, *amp;
  float *kx, *ky, *kz, *w, *xh, *xl, *yh, *yl, *zh, *zl;
  int cap;
};

// Tile shape of the whole-grid point x node kernels: 256 threads, each owning KP
// consecutive k-points of one (i, j) column; KCH k-chunks per tile.
struct TileShape { int kp, kch; };

// Generates the node list at time t into nb with one thread block; *d_count receives
// the total, *d_err the error bits (capacity / walk limit).
void th_launch_nodes(const DevProblem& P, double t, bool is_sol, const NodeBufView& nb, int* d_count, int* d_err,
                     cudaStream_t s);

// T at every grid point (p = i*ny*nz + j*nz + k) from the node list (custom points: every
// point, by the list kernels).
void th_launch_grid_sum(const DevProblem& P, const NodeBufView& nb, const int* d_count, double* d_T, int precision,
                        TileShape shape, unsigned long long* d_pairs, cudaStream_t s);

// T at n listed points (d_pts null: points 0 .. n - 1).
void th_launch_list_sum(const DevProblem& P, const NodeBufView& nb, const int* d_count, const int64_t* d_pts,
                        int64_t n, double* d_T, int precision, unsigned long long* d_pairs, cudaStream_t s);

// Converts the node list into the reference's 8 fields (expmod = log(amp)) in out[8][cap].
void th_launch_nodes_export(const NodeBufView& nb, const int* d_count, double* d_out, int cap, cudaStream_t s);

bool th_tile_shape_supported(TileShape shape);

// Tiles of one deck's grid for a tile shape.
int th_tile_count(const DevProblem& P, TileShape shape);

// Batched decks: node lists (one block per deck), then one persistent work-list grid over
// every deck's tiles (tile_off: exclusive prefix of tile counts, ndeck + 1 entries).
void th_launch_batch_nodes(int ndeck, const DevProblem* probs, const NodeBufView* views, const double* times,
                           int* counts, int* err, cudaStream_t s);
void th_launch_batch_grid(TileShape shape, int precision, const DevProblem* probs, const NodeBufView* views,
                          const int* counts, double* T, const long long* pnum_off, const int* tile_off, int ndeck,
                          int* ticket, unsigned long long* pairs, cudaStream_t s);
