/*
 * TEST INFRASTRUCTURE ONLY.  A thin C entry layer over the UNMODIFIED 3DThesis
 * library, compiled from the reference's own sources by oracle/Makefile (target
 * "ref") into oracle/_ref/.  It exists to pin the oracle and to generate the golden
 * fixtures under tests/golden/; nothing in the product or in the GPU-box tests loads it.
 *
 * Entry points call the reference's public interface:
 *   Init::GetFileNames / Init::ReadSimParams (src/Init.h), Grid (src/Grid.h),
 *   Calc::Integrate_Serial (src/Calc.h:23), Grid::Calc_T (src/Grid.h:290),
 *   Run::Simulate (src/Run.h), Grid::Output and Grid::Output_RRDF_csv (src/Grid.h), and
 *   the Grid getters (src/Grid.h:299-370).
 */
#include <cstdint>
#include <cstring>
#include <string>
#include <unistd.h>

#include "DataStructs.h"
#include "Grid.h"
#include "Init.h"
#include "Run.h"
#include "Calc.h"
#include "Util.h"

struct RefRun {
  Simdat sim;
  Grid* grid = nullptr;
};

extern "C" {

// Loads a deck the way bin/Main.cpp:44-77 does; the working directory becomes the
// deck's directory because the reference opens the files named in ParamInput.txt
// relative to the working directory.
void* ref_load(const char* deck_dir) {
  if (chdir(deck_dir) != 0) return nullptr;
  RefRun* r = new RefRun();
  r->sim.print = false;
  Init::GetFileNames(r->sim.files, "ParamInput.txt", r->sim.print);
  Init::ReadSimParams(r->sim);
  r->grid = new Grid(r->sim);
  r->sim.util.approxEndTime = r->sim.util.allScansEndTime;
  return r;
}

void ref_info(void* h, double* info) {
  RefRun* r = (RefRun*)h;
  info[0] = r->sim.domain.xnum; info[1] = r->sim.domain.ynum; info[2] = r->sim.domain.znum;
  info[3] = r->sim.domain.pnum; info[4] = (double)r->sim.beams.size();
  info[5] = (double)r->sim.param.SnapshotTimes.size(); info[6] = r->sim.util.allScansEndTime;
  info[7] = r->sim.settings.r_max;
}

double ref_snapshot_time(void* h, int i) { return ((RefRun*)h)->sim.param.SnapshotTimes.at(i); }

int ref_nodes(void* h, double t, int is_sol, double* out, int cap) {
  RefRun* r = (RefRun*)h;
  Nodes nodes;
  Calc::Integrate_Serial(nodes, r->sim, t, is_sol != 0);
  const int n = (int)nodes.size;
  const int m = n < cap ? n : cap;
  const vector<double>* f[8] = {&nodes.xb, &nodes.yb, &nodes.zb, &nodes.phix, &nodes.phiy, &nodes.phiz, &nodes.dtau, &nodes.expmod};
  for (int c = 0; c < 8; ++c) for (int i = 0; i < m; ++i) out[(size_t)c * cap + i] = (*f[c])[i];
  return n;
}

void ref_calc_T(void* h, double t, const int64_t* pts, int64_t n, double* T) {
  RefRun* r = (RefRun*)h;
  Nodes nodes;
  Calc::Integrate_Serial(nodes, r->sim, t, false);
  for (int64_t i = 0; i < n; ++i) T[i] = r->grid->Calc_T(t, nodes, r->sim, false, (int)pts[i]);
}

void ref_simulate(void* h) {
  RefRun* r = (RefRun*)h;
  Run::Simulate(*r->grid, r->sim);
}

// The reference's CSV writer for the grid's current state (Grid::Output, src/Grid.cpp:72-99),
// as bin/Main.cpp:104-108 calls it after a Solidification run: Data/<Name>.<name>.csv.
void ref_output(void* h, const char* name) {
  RefRun* r = (RefRun*)h;
  r->grid->Output(r->sim, name);
}

// The doubly reduced data a Stork run leaves in the grid (src/Grid.h:368-370): per row the
// cell index (3), the two step times (2) and the 16 vertex temperatures, in the run's order.
// Returns the row count; copies at most cap rows.
int64_t ref_rrdf(void* h, uint32_t* idx, double* ts, double* Ts, int64_t cap) {
  RefRun* r = (RefRun*)h;
  const vector<uint32_t>& I = r->grid->get_RRDF_idxs();
  const vector<double>& tt = r->grid->get_RRDF_ts();
  const vector<double>& TT = r->grid->get_RRDF_Ts();
  const int64_t n = (int64_t)tt.size() / 2;
  for (int64_t q = 0; q < n && q < cap; ++q) {
    for (int c = 0; c < 3; ++c) idx[3 * q + c] = I[3 * q + c];
    for (int c = 0; c < 2; ++c) ts[2 * q + c] = tt[2 * q + c];
    for (int c = 0; c < 16; ++c) Ts[16 * q + c] = TT[16 * q + c];
  }
  return n;
}

// The reference's RRDF writer (Grid::Output_RRDF_csv, src/Grid.cpp:203-238), as
// bin/Main.cpp:109-111 calls it after a Stork run: Data/<Name>.<name>.csv.
void ref_output_rrdf(void* h, const char* name) {
  RefRun* r = (RefRun*)h;
  r->grid->Output_RRDF_csv(r->sim, name);
}

// The temperature history file (Grid::Output_T_hist, src/Grid.cpp:101-174).
void ref_output_T_hist(void* h, const char* name) {
  RefRun* r = (RefRun*)h;
  r->grid->Output_T_hist(r->sim, name);
}

// The same rows as the reference's binary file (Grid::Output_RRDF_bin, src/Grid.cpp:241-273).
void ref_output_rrdf_bin(void* h, const char* name) {
  RefRun* r = (RefRun*)h;
  r->grid->Output_RRDF_bin(r->sim, name);
}

// The reduced data a run with Output RDF 1 leaves in the grid (Grid::get_RDF_tm / _tl /
// _cr, src/Grid.h:360-362): per point the three counts, then all values in point order
// (per point its tm, then tl, then cr values).  Returns the number of values; copies at most
// cap.
int64_t ref_rdf(void* h, int32_t* counts, double* vals, int64_t cap) {
  RefRun* r = (RefRun*)h;
  Grid& g = *r->grid;
  int64_t n = 0;
  for (int p = 0; p < r->sim.domain.pnum; ++p) {
    const vector<double> v[3] = {g.get_RDF_tm(p), g.get_RDF_tl(p), g.get_RDF_cr(p)};
    for (int c = 0; c < 3; ++c) {
      if (counts) counts[3 * p + c] = (int32_t)v[c].size();
      for (double x : v[c]) { if (vals && n < cap) vals[n] = x; ++n; }
    }
  }
  return n;
}

// The reference's RDF writer (Grid::Output_RDF, src/Grid.cpp:176-201), as bin/Main.cpp:117
// calls it: Data/<Name>.<name>.csv.
void ref_output_rdf(void* h, const char* name) {
  RefRun* r = (RefRun*)h;
  r->grid->Output_RDF(r->sim, name);
}

int ref_field(void* h, const char* name, double* out) {
  RefRun* r = (RefRun*)h;
  Grid& g = *r->grid;
  const std::string f(name);
  const int n = r->sim.domain.pnum;
  for (int p = 0; p < n; ++p) {
    double v;
    if (f == "T") v = g.get_T(p);
    else if (f == "tSol") v = g.get_tSol(p);
    else if (f == "G") v = g.get_G(p);
    else if (f == "V") v = g.get_V(p);
    else if (f == "Gx") v = g.get_Gx(p);
    else if (f == "Gy") v = g.get_Gy(p);
    else if (f == "Gz") v = g.get_Gz(p);
    else if (f == "dTdt") v = g.get_dTdt(p);
    else if (f == "eqFrac") v = g.get_eqFrac(p);
    else if (f == "numMelt") v = g.get_numMelt(p);
    else if (f == "depth") v = g.get_depth(p);
    else if (f == "output_flag") v = g.get_output_flag(p) ? 1.0 : 0.0;
    else return 2;
    out[p] = v;
  }
  return 0;
}

}  // extern "C"
