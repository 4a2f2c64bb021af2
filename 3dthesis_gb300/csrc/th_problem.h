// Problem description shared by the host driver and the device kernels.
//
// HostProblem is the parsed deck (the reference's Simdat, src/DataStructs.h:163-183);
// DevProblem is the read-only view every kernel receives by value.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#define TH_MAX_BEAMS 16
#define TH_MAX_IMAGES 64

enum { TH_TRACK_NONE = 0, TH_TRACK_VOLUME = 1, TH_TRACK_SURFACE = 2, TH_TRACK_STORK = 3 };

// One path segment (src/DataStructs.h:42-48): end point, power modulation, speed or dwell,
// end time.  mode 0 = line, 1 = spot.
struct DevSeg {
  double x, y, z, q, prm, tend;
  double rt0;               // line segments: 0.58870501125 * ax / speed of the beam that scans it
  int32_t mode, pad;
};

struct DevBeam {
  double ax, ay, az;        // Gaussian widths (m)
  double ax2, ay2, az2;     // ax*ax etc.
  double nond;              // ax^2 / a
  double beta;              // (3/pi)^1.5 * q / (rho c)
  double tlast;             // end time of this beam's path
  double tsub;              // beam-trace look-back (CheckRadius^2 - 1) ax^2 / (12 a)
  double r2;                // beam-trace radius squared, CheckRadius^2 ax^2
  int32_t seg_off, nseg;    // segments [seg_off, seg_off + nseg) of DevProblem::segs
};

struct DevProblem {
  const DevSeg* segs;
  int32_t nbeams;
  DevBeam beam[TH_MAX_BEAMS];
  // material
  double T0, TL, a, a12;    // a12 = 12 * a
  float tl_df[3];           // TL - T0 as three floats (hi + mid + lo), for the FP32 tracking's liquid test
  double cetN0, cetn, ceta;
  // domain
  int32_t nx, ny, nz;       // axis counts
  // floor(x / nz) and floor(x / ny) as (x * m) >> s for 0 <= x < 2^31 (point and column ids)
  uint32_t div_nz_m, div_ny_m;
  int32_t div_nz_s, div_ny_s;
  int32_t gx, gy, gz;       // the same truncated to uint16_t (the reference grid's width)
  int64_t pnum;
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double xres, yres, zres;  // domain resolution used by the beam trace
  double hx, hy, hz;        // point spacing used for coordinates: (max - min) / (g - 1)
  double rx0, rx1, ry0, ry1;// domain +- r_max (power cut-off box)
  // boundary images: (cx, cy, cz) per image, image 0 = identity
  int32_t n_images;
  int32_t img[TH_MAX_IMAGES][3];
  double bcx0, bcx1, bcy0, bcy1, bcz0, bcz1;
  // solidification
  double dt, sol_tol;
  int32_t sol_iter;
  int32_t tracking;
  int32_t compress;         // path compression (GaussCompressIntegrate) on
  double rcheck;
  double end_time;
  // Gauss-Legendre tables for orders 2/4/8/16 packed at offset order - 2
  double gl_loc[30], gl_w[30];
  // custom points (Domain: Custom File): every point's coordinates, pnum each (device
  // arrays); null for a grid
  const double* cx;
  const double* cy;
  const double* cz;
};

struct HostBeam { double ax, ay, az, eff, q, nond, power; };

struct HostProblem {
  std::string dir, name;
  // material
  double T0, TL, kon, cps, rho, a, cetN0, cetn, ceta;
  std::vector<HostBeam> beams;
  std::vector<std::vector<DevSeg>> paths;
  // domain
  int nx, ny, nz;
  int64_t pnum;
  double xmin, xmax, ymin, ymax, zmin, zmax, xres, yres, zres;
  bool use_bcs;
  bool compress;                  // path compression (Settings: Path Compression)
  int bc_refl;
  double bcx0, bcx1, bcy0, bcy1, bcz0;
  // mode
  int mode;                       // 0 Snapshots, 1 Solidification
  std::vector<double> snaps;
  int tracking;
  double dt;
  int out_freq;
  double rcheck;
  // outputs
  bool o_x, o_y, o_z, o_T, o_tSol, o_G, o_Gx, o_Gy, o_Gz, o_V, o_dTdt, o_eqFrac, o_depth, o_numMelt;
  bool o_rdf;                     // the reduced data format (per point melting / solidification events)
  bool o_T_hist;                  // every point's temperature at every evaluation (Tracking None)
  bool custom = false;            // points from a points file (Domain: Custom File), not a grid
  std::vector<double> px, py, pz; // their coordinates (m)
  bool do_sol;
  // settings
  double sol_tol;
  int sol_iter;
  double t_hist, p_hist, r_max;
  double end_time;
};

// Parses a deck (ParamInput.txt and the files it names).  Returns false with a message.
bool th_load_deck(const std::string& param_input, HostProblem& hp, std::string& err);

// Builds the device view; the caller supplies the device address of the packed segments.
void th_make_dev_problem(const HostProblem& hp, const DevSeg* d_segs, DevProblem& dp);

// Packs every path's segments into one array (the order DevBeam::seg_off indexes).
std::vector<DevSeg> th_pack_segments(const HostProblem& hp);

// Gauss-Legendre abscissae / weights rounded to 8 decimals, orders 2, 4, 8, 16.
void th_gauss_tables(double loc[30], double w[30]);
