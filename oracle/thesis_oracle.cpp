/*
 * TEST INFRASTRUCTURE ONLY - the parity oracle and CPU baseline for the GPU build.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU legs load this library.
 *
 * A double-precision CPU restatement of 3DThesis's hot path, written from the
 * reference's behaviour (file:line citations below are relative to the 3DThesis
 * source tree).  Operation order inside every floating-point expression follows the
 * reference so that the oracle reproduces it to the last few ulps; the oracle is
 * compiled with -ffp-contract=off so x86-64 and aarch64 builds agree.
 *
 * Deliberate, documented differences from the reference:
 *  - The segment search (src/Calc.cpp:99-104) keeps a function-static hint that is
 *    shared between threads.  Here the search is stateless: the first segment s>=1
 *    with t <= seg_time[s], clamped to the last one.  For a non-decreasing sequence of
 *    times (every driver loop) this is exactly the reference's answer; the two can
 *    differ only when t equals a segment end time bit-for-bit after a later time was
 *    searched.
 *  - Integrate_Parallel (src/Calc.cpp:21-46) precomputes nodes at t_k + i*dt for
 *    MaxThreads > 1.  The oracle always uses the driver's accumulated t (the
 *    reference's MaxThreads = 1 behaviour).
 */
#include "thesis_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cctype>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include <omp.h>

namespace {

const double kPi = 3.14159265358979323846;   // src/DataStructs.h:25

struct Seg { int mode; double x, y, z, q, prm, tend; };
struct Beam { double ax, ay, az, eff, q, nond; };

struct Nodes {
  std::vector<double> xb, yb, zb, ipx, ipy, ipz, dtau, expmod;
  size_t size() const { return xb.size(); }
  void clear() { xb.clear(); yb.clear(); zb.clear(); ipx.clear(); ipy.clear(); ipz.clear(); dtau.clear(); expmod.clear(); }
};

// Gauss-Legendre abscissae/weights for orders 2, 4, 8, 16 (packed at offset order-2),
// rounded to 8 decimal places as the reference's tables are (src/Calc.cpp:72-86).
struct GaussTables {
  double loc[30], w[30];
  GaussTables() {
    const int orders[4] = {2, 4, 8, 16};
    for (int oi = 0; oi < 4; ++oi) {
      const int n = orders[oi];
      const int base = n - 2;
      for (int i = 0; i < n; ++i) {
        // i-th root in ascending order: start from the Chebyshev guess of root n-i
        double x = std::cos(kPi * ((n - i) - 0.25) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; ++it) {
          double p0 = 1.0, p1 = x;
          for (int k = 2; k <= n; ++k) { double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = p2; }
          dp = n * (x * p1 - p0) / (x * x - 1.0);
          double dx = p1 / dp;
          x -= dx;
          if (std::fabs(dx) < 1e-17) break;
        }
        double p0 = 1.0, p1 = x;
        for (int k = 2; k <= n; ++k) { double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k; p0 = p1; p1 = p2; }
        dp = n * (x * p1 - p0) / (x * x - 1.0);
        const double wt = 2.0 / ((1.0 - x * x) * dp * dp);
        loc[base + i] = std::round(x * 1e8) / 1e8;
        w[base + i] = std::round(wt * 1e8) / 1e8;
      }
    }
  }
};
const GaussTables& gauss() { static GaussTables g; return g; }

enum { TRACK_NONE = 0, TRACK_VOLUME = 1, TRACK_SURFACE = 2, TRACK_STORK = 3 };

struct Problem {
  std::string dir;
  // material (src/DataStructs.h:63-71)
  double T0, TL, kon, cps, rho, a, cetN0, cetn, ceta;
  std::vector<Beam> beams;
  std::vector<std::vector<Seg>> paths;
  // domain (src/DataStructs.h:98-122)
  int nx, ny, nz; long pnum;
  double xmin, xmax, ymin, ymax, zmin, zmax, xres, yres, zres;
  bool use_bcs; int bc_refl; double bcx0, bcx1, bcy0, bcy1, bcz0;
  // grid copies of the axis counts are uint16_t in the reference (src/Grid.h:65-67)
  int gx, gy, gz;
  // custom points in place of a grid (Domain: Custom File, src/Init.cpp:686-703): their
  // coordinates, in the file's order
  bool custom = false;
  std::vector<double> cx, cy, cz;
  // mode
  int mode;  // 0 Snapshots, 1 Solidification
  std::vector<double> snaps;
  int tracking; double dt; int out_freq; double rcheck; bool secondary;
  // outputs
  bool o_T, o_tSol, o_G, o_Gx, o_Gy, o_Gz, o_V, o_dTdt, o_eqFrac, o_depth, o_numMelt;
  bool o_rdf = false;       // the reduced data format: per point its melt events (src/Grid.h:103-105)
  // settings
  double sol_tol; int sol_iter; double t_hist, p_hist, r_max; int compress; int thnum;
  double end_time;
  bool do_sol;
  mutable bool walk_error = false;   // a compressed walk met a segment end outside the r_max box
  // grid state
  std::vector<double> T, T_last, tSol, G, V, Gx, Gy, Gz, dTdt, eqFrac, depth;
  // per point, for the parity tests' explanations: the closest approach of an evaluated T
  // to T_L (DBL_MAX: never evaluated) and the secant's T - T_last at its latest
  // solidification (0: never solidified)
  std::vector<double> band, sol_dT;
  // RDF (Output RDF 1): per point the melting times (pushed by Surface tracking's reset
  // sweep, src/Run.cpp:604-609), solidification times and cooling rates (Grid::Solidify,
  // src/Grid.cpp:322,547), and per solidification its secant's T - T_last (for tests)
  std::vector<std::vector<double>> rdf_tm, rdf_tl, rdf_cr, rdf_dT;
  // Stork's doubly reduced data (src/Run.cpp:711-1079): per output cell its index (i, j, k),
  // the two step times and the 16 vertex temperatures (8 at the earlier time, then 8 at the
  // later one)
  std::vector<uint32_t> rrdf_idx;
  std::vector<double> rrdf_t, rrdf_T;
  std::vector<int> numMelt;
  std::vector<unsigned char> calc, outflag;
  std::atomic<long long> pairs{0};
};

// ------------------------------------------------------------------ input layer
struct Tok { std::string s; int line; };

bool tokenize(const std::string& file, std::vector<Tok>& toks) {
  std::ifstream in(file.c_str());
  if (!in.is_open()) return false;
  std::string line; int ln = 0;
  while (std::getline(in, line)) {
    size_t i = 0;
    while (i < line.size()) {
      while (i < line.size() && std::isspace((unsigned char)line[i])) ++i;
      size_t j = i;
      while (j < line.size() && !std::isspace((unsigned char)line[j])) ++j;
      if (j > i) toks.push_back({line.substr(i, j - i), ln});
      i = j;
    }
    ++ln;
  }
  return true;
}

size_t next_line(const std::vector<Tok>& t, size_t i) {
  const int ln = t[i].line;
  while (i < t.size() && t[i].line == ln) ++i;
  return i;
}

// Brace-block keyword reader: src/Init.cpp:77-131 (first token of a line names a block,
// the next token must be "{", then "key value" pairs, one per line, until "}").
bool read_blocks(const std::string& file, const std::vector<std::string>& mains,
                 const std::vector<std::vector<std::string>>& subs,
                 std::vector<std::vector<std::string>>& vals, std::vector<int>* counts = nullptr) {
  vals.assign(mains.size(), {});
  for (size_t m = 0; m < mains.size(); ++m) vals[m].assign(subs[m].size(), "");
  if (counts) counts->assign(mains.size(), 0);
  std::vector<Tok> t;
  if (!tokenize(file, t)) return false;
  size_t i = 0;
  while (i < t.size()) {
    const std::string w = t[i].s;
    i = next_line(t, i);
    int mi = -1;
    for (size_t m = 0; m < mains.size(); ++m) if (w == mains[m]) { mi = (int)m; break; }
    if (mi < 0) continue;
    if (counts) (*counts)[mi]++;
    if (i >= t.size()) break;
    const std::string br = t[i].s;
    i = next_line(t, i);
    if (br != "{") continue;
    while (i < t.size()) {
      const std::string key = t[i].s;
      if (key == "}") { i = next_line(t, i); break; }
      if (i + 1 >= t.size()) { i = t.size(); break; }
      const std::string v = t[i + 1].s;
      i = next_line(t, i + 1);
      for (size_t s = 0; s < subs[mi].size(); ++s) if (key == subs[mi][s]) vals[mi][s] = v;
    }
  }
  return true;
}

double dval(const std::string& s, double def) { return s.empty() ? def : std::stod(s); }
int ival(const std::string& s, int def) { return s.empty() ? def : std::stoi(s); }

std::string resolve(const std::string& dir, const std::string& f) {
  if (f.empty() || f[0] == '/') return f;
  return dir + "/" + f;
}

// '*' wildcard expands to 1, 2, ... until a file is missing (src/Init.cpp:445-487).
std::vector<std::string> expand(const std::string& pattern) {
  std::vector<std::string> out;
  size_t pos = pattern.find('*');
  if (pos == std::string::npos) { out.push_back(pattern); return out; }
  for (int n = 1;; ++n) {
    std::string f = pattern.substr(0, pos) + std::to_string(n) + pattern.substr(pos + 1);
    std::ifstream in(f.c_str());
    if (!in.is_open()) break;
    out.push_back(f);
  }
  return out;
}

// Path file: header line, then "mode x y z pmod param" in mm; implicit origin spot;
// segment end times from speed or dwell (src/Init.cpp:560-625).
bool read_path(const std::string& file, std::vector<Seg>& path) {
  std::ifstream in(file.c_str());
  path.clear();
  path.push_back({1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0});
  if (!in.is_open()) return false;
  std::string header;
  std::getline(in, header);
  while (true) {                     // one record per line; the rest of the line is ignored
    Seg s{1, 0, 0, 0, 0, 0, 0};
    if (!(in >> s.mode >> s.x >> s.y >> s.z >> s.q >> s.prm)) break;
    s.x *= 1e-3; s.y *= 1e-3; s.z *= 1e-3;
    path.push_back(s);
    std::string rest;
    if (!std::getline(in, rest)) break;
  }
  path[0].tend = 0.0;
  for (size_t k = 1; k < path.size(); ++k) {
    if (path[k].mode) path[k].tend = path[k - 1].tend + path[k].prm;
    else {
      const double dx = path[k].x - path[k - 1].x, dy = path[k].y - path[k - 1].y, dz = path[k].z - path[k - 1].z;
      const double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
      path[k].tend = path[k - 1].tend + dist / path[k].prm;
    }
  }
  return true;
}

bool load_problem(Problem& P, const std::string& param_input, std::string& err) {
  size_t sl = param_input.find_last_of('/');
  P.dir = (sl == std::string::npos) ? "." : param_input.substr(0, sl);
  std::vector<std::vector<std::string>> v;
  if (!read_blocks(param_input, {"Simulation", "Options"},
                   {{"Name", "Mode", "Material", "Beam", "Path"}, {"Domain", "Output", "Settings"}}, v)) {
    err = "cannot open " + param_input; return false;
  }
  const std::string f_mode = resolve(P.dir, v[0][1]), f_mat = resolve(P.dir, v[0][2]),
                    f_beam = resolve(P.dir, v[0][3]), f_path = resolve(P.dir, v[0][4]),
                    f_dom = resolve(P.dir, v[1][0]), f_out = resolve(P.dir, v[1][1]),
                    f_set = resolve(P.dir, v[1][2]);
  if (v[0][1].empty() || v[0][3].empty() || v[0][4].empty()) { err = "mode, beam and path files are required"; return false; }

  // beams (src/Init.cpp:488-515, 862-865)
  for (const std::string& bf : expand(f_beam)) {
    std::vector<std::vector<std::string>> b;
    read_blocks(bf, {"Shape", "Intensity"}, {{"Width_X", "Width_Y", "Depth_Z"}, {"Power", "Efficiency"}}, b);
    Beam B;
    B.ax = dval(b[0][0], 10.0e-6); B.ay = dval(b[0][1], 10.0e-6); B.az = dval(b[0][2], 1.0e-6);
    B.q = dval(b[1][0], 1200); B.eff = dval(b[1][1], 1.0);
    if (B.eff == DBL_MAX) B.eff = 1.0;
    B.q = B.q * B.eff * 2.0;
    P.beams.push_back(B);
  }
  // material (src/Init.cpp:410-443, 859-861)
  {
    std::vector<std::vector<std::string>> m;
    read_blocks(f_mat, {"Constants", "CET"}, {{"T_0", "T_L", "k", "c", "p"}, {"N0", "n", "a"}}, m);
    P.T0 = dval(m[0][0], 1273.0); P.TL = dval(m[0][1], 1610.0); P.kon = dval(m[0][2], 26.6);
    P.cps = dval(m[0][3], 600.0); P.rho = dval(m[0][4], 7451.0);
    P.cetN0 = dval(m[1][0], DBL_MAX); P.cetn = dval(m[1][1], DBL_MAX); P.ceta = dval(m[1][2], DBL_MAX);
    P.a = P.kon / (P.rho * P.cps);
  }
  for (Beam& B : P.beams) B.nond = B.ax * B.ax / P.a;      // src/Util.cpp:138-143
  // paths
  for (const std::string& pf : expand(f_path)) {
    std::vector<Seg> path;
    read_path(pf, path);
    P.paths.push_back(path);
  }
  if (P.paths.empty() || P.paths.size() != P.beams.size()) { err = "beam and path counts differ"; return false; }
  for (auto& path : P.paths) if (path.size() < 2) { err = "path has no segments"; return false; }
  P.end_time = 0.0;
  for (auto& path : P.paths) P.end_time = std::max(P.end_time, path.back().tend);

  // mode (src/Init.cpp:305-408)
  {
    std::vector<std::vector<std::string>> tmp; std::vector<int> cnt;
    read_blocks(f_mode, {"Snapshots", "Solidification"}, {{}, {}}, tmp, &cnt);
    if (cnt[0] + cnt[1] != 1) { err = "mode file must name exactly one mode"; return false; }
    if (cnt[0]) {
      P.mode = 0;
      std::vector<std::vector<std::string>> m;
      read_blocks(f_mode, {"Snapshots"}, {{"Times", "ScanFracs", "Tracking"}}, m);
      if (!m[0][0].empty() && !m[0][1].empty()) { err = "too many time types"; return false; }
      std::string item;
      if (!m[0][0].empty()) { std::stringstream ss(m[0][0]); while (std::getline(ss, item, ',')) P.snaps.push_back(std::stod(item)); }
      if (!m[0][1].empty()) { std::stringstream ss(m[0][1]); while (std::getline(ss, item, ',')) P.snaps.push_back(std::stod(item) / 100.0 * P.end_time); }
      const std::string tr = m[0][2].empty() ? "None" : m[0][2];
      // other modes are refused once the domain is read: custom points go without tracking
      // (src/Run.cpp:61)
      P.tracking = tr == "None" ? TRACK_NONE : -1;
      P.dt = 1e-5; P.out_freq = INT_MAX; P.rcheck = 1.0; P.secondary = false;
    } else {
      P.mode = 1;
      std::vector<std::vector<std::string>> m;
      read_blocks(f_mode, {"Solidification"}, {{"Tracking", "Timestep", "OutputFrequency", "CheckRadius", "Secondary"}}, m);
      const std::string tr = m[0][0].empty() ? "None" : m[0][0];
      P.tracking = tr == "Volume" ? TRACK_VOLUME : tr == "Surface" ? TRACK_SURFACE : tr == "Stork" ? TRACK_STORK
                                                                                                   : TRACK_NONE;
      if (!(tr == "None" || tr == "Volume" || tr == "Surface" || tr == "Stork")) { err = "unsupported tracking " + tr; return false; }
      P.dt = dval(m[0][1], 1e-5); P.out_freq = ival(m[0][2], INT_MAX);
      P.rcheck = dval(m[0][3], 1.0); P.secondary = m[0][4].empty() ? false : (bool)std::stoi(m[0][4]);
      if (P.secondary) { err = "secondary solidification is not supported"; return false; }
    }
  }
  // domain (src/Init.cpp:627-707), scan bounds (src/Util.cpp:82-136), params (src/Init.cpp:866-908)
  {
    std::vector<std::vector<std::string>> d;
    read_blocks(f_dom, {"X", "Y", "Z", "BoundaryConditions", "Custom"},
                {{"Min", "Max", "Num", "Res"}, {"Min", "Max", "Num", "Res"}, {"Min", "Max", "Num", "Res"},
                 {"X_min", "X_max", "Y_min", "Y_max", "Z_min", "Reflections"}, {"File"}}, d);
    P.xmin = dval(d[0][0], -DBL_MAX); P.xmax = dval(d[0][1], DBL_MAX); P.nx = ival(d[0][2], INT_MAX); P.xres = dval(d[0][3], 50e-6);
    P.ymin = dval(d[1][0], -DBL_MAX); P.ymax = dval(d[1][1], DBL_MAX); P.ny = ival(d[1][2], INT_MAX); P.yres = dval(d[1][3], 50e-6);
    P.zmin = dval(d[2][0], -DBL_MAX); P.zmax = dval(d[2][1], DBL_MAX); P.nz = ival(d[2][2], INT_MAX); P.zres = dval(d[2][3], 50e-6);
    P.bcx0 = dval(d[3][0], DBL_MAX); P.bcx1 = dval(d[3][1], DBL_MAX); P.bcy0 = dval(d[3][2], DBL_MAX);
    P.bcy1 = dval(d[3][3], DBL_MAX); P.bcz0 = dval(d[3][4], DBL_MAX); P.bc_refl = ival(d[3][5], INT_MAX);
    P.use_bcs = P.bcx0 != DBL_MAX || P.bcx1 != DBL_MAX || P.bcy0 != DBL_MAX || P.bcy1 != DBL_MAX || P.bcz0 != DBL_MAX;
    // custom points, read as Init::FileRead_Points does (src/Init.cpp:816-857): the first
    // line is skipped; then, point by point, the rest of the current line is skipped and
    // three numbers are read (mm), until a read fails
    P.custom = !d[4][0].empty();
    if (P.custom) {
      std::ifstream in(resolve(P.dir, d[4][0]));
      if (!in) { err = "cannot open the points file"; return false; }
      std::string line;
      double x = 0, y = 0, z = 0;
      while (std::getline(in, line) && (in >> x >> y >> z)) {
        P.cx.push_back(x / 1000.0); P.cy.push_back(y / 1000.0); P.cz.push_back(z / 1000.0);
      }
      if (P.cx.empty()) { err = "no points in the points file"; return false; }
    }

    double sx0 = DBL_MAX, sx1 = -DBL_MAX, sy0 = DBL_MAX, sy1 = -DBL_MAX, sz0 = DBL_MAX, sz1 = -DBL_MAX;
    double px = 0, py = 0, pz = 0, pq = 0; bool first = true;
    for (auto& path : P.paths) for (auto& s : path) {
      if (s.q > 0.0) {
        if (first) { sx0 = sx1 = s.x; sy0 = sy1 = s.y; sz0 = sz1 = s.z; }
        else {
          sx0 = std::min(sx0, s.x); sx1 = std::max(sx1, s.x); sy0 = std::min(sy0, s.y); sy1 = std::max(sy1, s.y);
          sz0 = std::min(sz0, s.z); sz1 = std::max(sz1, s.z);
          if (pq == 0.0 && s.mode == 0) {
            sx0 = std::min(sx0, px); sx1 = std::max(sx1, px); sy0 = std::min(sy0, py); sy1 = std::max(sy1, py);
            sz0 = std::min(sz0, pz); sz1 = std::max(sz1, pz);
          }
        }
      }
      first = false; px = s.x; py = s.y; pz = s.z; pq = s.q;
    }
    if (P.xmin == -DBL_MAX) P.xmin = sx0 - 500e-6;
    if (P.xmax == DBL_MAX) P.xmax = sx1 + 500e-6;
    if (P.ymin == -DBL_MAX) P.ymin = sy0 - 500e-6;
    if (P.ymax == DBL_MAX) P.ymax = sy1 + 500e-6;
    if (P.zmin == -DBL_MAX) P.zmin = sz0 - 250e-6;
    if (P.zmax == DBL_MAX) P.zmax = sz1;

    if (P.custom) {                   // no grid (src/Init.cpp:866-869), and no tracking (src/Run.cpp:61, 391)
      P.nx = (int)P.cx.size(); P.ny = P.nz = 1;
      P.pnum = (long)P.cx.size();
      P.gx = P.gy = P.gz = 1;
      P.tracking = TRACK_NONE;
    } else {
      if (P.tracking < 0) { err = "snapshot tracking modes other than None are not supported"; return false; }
      if (P.nx == INT_MAX) { P.nx = 1 + int(0.5 + (P.xmax - P.xmin) / P.xres); P.xmax = P.xmin + (P.nx - 1) * P.xres; }
      else if (P.nx != 1) P.xres = (P.xmax - P.xmin) / (P.nx - 1);
      else P.xres = DBL_MAX;
      if (P.ny == INT_MAX) { P.ny = 1 + int(0.5 + (P.ymax - P.ymin) / P.yres); P.ymax = P.ymin + (P.ny - 1) * P.yres; }
      else if (P.ny != 1) P.yres = (P.ymax - P.ymin) / (P.ny - 1);
      else P.yres = DBL_MAX;
      if (P.nz == INT_MAX) { P.nz = 1 + int(0.5 + (P.zmax - P.zmin) / P.zres); P.zmax = P.zmin + (P.nz - 1) * P.zres; }
      else if (P.ny != 1) P.zres = (P.zmax - P.zmin) / (P.nz - 1);   // the reference tests ynum here
      else P.zres = DBL_MAX;
      if (P.nx <= 0 || P.ny <= 0 || P.nz <= 0 || P.nx > 65535 || P.ny > 65535 || P.nz > 65535) { err = "grid size out of range"; return false; }
      P.pnum = (long)P.nx * P.ny * P.nz;
      P.gx = (uint16_t)P.nx; P.gy = (uint16_t)P.ny; P.gz = (uint16_t)P.nz;
    }
  }
  // outputs (src/Init.cpp:709-771)
  {
    std::vector<std::vector<std::string>> o;
    read_blocks(f_out, {"Grid", "Temperature", "Solidification", "Solidification+"},
                {{"x", "y", "z"}, {"T", "T_hist"},
                 {"tSol", "G", "Gx", "Gy", "Gz", "V", "dTdt", "eqFrac", "depth", "numMelt", "RDF", "MP_Stats"},
                 {"H", "Hx", "Hy", "Hz"}}, o);
    auto b = [](const std::string& s, bool def) { return s.empty() ? def : (bool)std::stoi(s); };
    P.o_T = b(o[1][0], true);
    P.o_tSol = b(o[2][0], false); P.o_G = b(o[2][1], false); P.o_Gx = b(o[2][2], false); P.o_Gy = b(o[2][3], false);
    P.o_Gz = b(o[2][4], false); P.o_V = b(o[2][5], false); P.o_dTdt = b(o[2][6], false); P.o_eqFrac = b(o[2][7], false);
    P.o_depth = b(o[2][8], false); P.o_numMelt = b(o[2][9], false); P.o_rdf = b(o[2][10], false);
    // every solidification output, RDF too, turns the solidification fields on (src/Grid.h:180-241)
    P.do_sol = P.mode == 1 && (P.o_tSol || P.o_G || P.o_V || P.o_Gx || P.o_Gy || P.o_Gz || P.o_dTdt || P.o_eqFrac ||
                               P.o_rdf);
  }
  // settings (src/Init.cpp:772-814) and r_max (src/Util.cpp:145-166)
  {
    std::vector<std::vector<std::string>> s;
    read_blocks(f_set, {"Temperature", "Path", "Compute", "MPI"},
                {{"Sol_Tol", "Sol_Iter", "Cutoff_Peak", "Cutoff_T0TL"}, {"Buffer", "Compression"}, {"MaxThreads", "PINT"}, {"Overlap"}}, s);
    P.sol_tol = dval(s[0][0], 1e-3); P.sol_iter = ival(s[0][1], 10);
    P.t_hist = dval(s[0][2], 1e-9); P.p_hist = dval(s[0][3], 1e-2);
    P.r_max = dval(s[1][0], -1.0); P.compress = ival(s[1][1], 0);
    P.thnum = ival(s[2][0], 1);

    P.t_hist = 1.0 / P.t_hist;
    if (P.r_max < 0.0) {
      for (const Beam& B : P.beams) {
        if (P.t_hist < std::exp(3.0 / 2.0)) P.r_max = B.ax * std::sqrt(std::log(P.t_hist) / 3.0);
        else P.r_max = B.ax * std::pow(P.t_hist, (1.0 / 3.0)) / std::sqrt(2.0 * std::exp(1.0));
        const double beta = std::pow(3.0 / 3.14159, 1.5) * B.q / (P.rho * P.cps);
        const double x = (P.TL - P.T0) * P.p_hist;
        double r2;
        if (beta / (x * B.ax * B.ax * B.ax) < std::exp(3.0 / 2.0)) r2 = B.ax * std::sqrt(std::log(beta / (x * B.ax * B.ax * B.ax)) / 3.0);
        else r2 = std::pow(beta / x, (1.0 / 3.0)) / std::sqrt(2.0 * std::exp(1.0));
        P.r_max = std::max(P.r_max, r2);
      }
    }
  }
  return true;
}

// ------------------------------------------------------------------ nodes
inline bool in_rmax(const Problem& P, double x, double y) {                 // src/Util.cpp:168-172
  if ((x > (P.xmax + P.r_max)) || (x < (P.xmin - P.r_max))) return false;
  if ((y > (P.ymax + P.r_max)) || (y < (P.ymin - P.r_max))) return false;
  return true;
}

struct Loc { double x, y, z, q; };
inline Loc beam_loc(const Problem& P, const std::vector<Seg>& path, double t, int s) {   // src/Util.cpp:211-237
  Loc L;
  if (path[s].mode) { L.x = path[s].x; L.y = path[s].y; L.z = path[s].z; }
  else {
    const double dx = path[s].x - path[s - 1].x, dy = path[s].y - path[s - 1].y, dz = path[s].z - path[s - 1].z;
    const double tc = t - path[s - 1].tend, span = path[s].tend - path[s - 1].tend;
    L.x = path[s - 1].x + (tc / span) * dx;
    L.y = path[s - 1].y + (tc / span) * dy;
    L.z = path[s - 1].z + (tc / span) * dz;
  }
  L.q = in_rmax(P, L.x, L.y) ? path[s].q : 0.0;
  return L;
}

inline double ref_time(const std::vector<Seg>& path, const Beam& B, double tpp, int s) {   // src/Util.cpp:192-209
  const double spp = std::max(tpp / B.nond, 0.0);
  if (path[s].mode == 0) { const double t0 = 0.58870501125 * B.ax / path[s].prm; return t0 * std::sqrt(12.0 * spp + 1.0); }
  double r = path[s].tend - path[s - 1].tend;
  if (r == 0) r = 1.0e-9;
  return r;
}

inline void add_node(Nodes& N, double x, double y, double z, double phx, double phy, double phz, double dtau, double qb) {
  N.xb.push_back(x); N.yb.push_back(y); N.zb.push_back(z);                  // src/Util.cpp:40-50
  N.ipx.push_back(1.0 / phx); N.ipy.push_back(1.0 / phy); N.ipz.push_back(1.0 / phz);
  N.dtau.push_back(dtau);
  N.expmod.push_back(std::log(qb) - std::log(phx * phy * phz) / 2.0);
}

int find_seg(const std::vector<Seg>& path, double t) {
  int s = 1;
  while (t > path[s].tend && s + 1 < (int)path.size()) ++s;
  return s;
}

// FNV-1a over 64-bit words: the signature of a walk's discrete choices.
inline void sig_mix(uint64_t* h, uint64_t v) {
  if (!h) return;
  for (int i = 0; i < 8; ++i) { *h ^= (v >> (8 * i)) & 0xffu; *h *= 1099511628211ull; }
}

// Adaptive Gauss integration back along every beam's path (src/Calc.cpp:67-211).  With
// sig, also hashes every discrete choice of the walk - per beam the starting segment, per
// interval its segment, the number of step-cap doublings so far, its Gauss order and
// whether it was cut at the segment's start, and per candidate node whether it was kept -
// so that two times with equal signatures have node lists that are the same continuous
// function of t.
void gauss_nodes(const Problem& P, double t, bool is_sol, Nodes& N, uint64_t* sig = nullptr) {
  const GaussTables& G = gauss();
  for (size_t b = 0; b < P.paths.size(); ++b) {
    const Beam& B = P.beams[b];
    const std::vector<Seg>& path = P.paths[b];
    int s = find_seg(path, t);
    sig_mix(sig, 0xbea0000000000000ull | (uint64_t)b);
    sig_mix(sig, (uint64_t)s);
    const double beta = std::pow(3.0 / kPi, 1.5) * B.q / (P.rho * P.cps);
    const double t0 = 0.0;                               // src/Util.cpp:174-190 always returns 0
    double step0 = B.nond;
    if (is_sol) step0 *= B.az;
    double stepmax = step0;
    int order = 16;
    {
      Loc L = beam_loc(P, path, t, s);
      const double qb = L.q * beta;
      const bool keep = t <= path.back().tend && qb > 0.0;
      sig_mix(sig, keep ? 1u : 0u);
      if (keep) add_node(N, L.x, L.y, L.z, B.ax * B.ax + 0.0, B.ay * B.ay + 0.0, B.az * B.az + 0.0, 0.0, qb);
    }
    double t2 = t, t1 = t, tpp = 0.0;
    int ndbl = 0;                                        // doublings of the step cap so far
    if (t > path.back().tend) { tpp += t - path.back().tend; t2 = path.back().tend; }
    while (tpp >= 2 * stepmax - step0) { stepmax *= 2.0; ++ndbl; if (order != 2) order /= 2; }
    bool more = true;
    while (more) {
      bool sw = false;
      const double rt = ref_time(path, B, tpp, s);
      const double use = (rt < stepmax) ? rt : stepmax;
      t1 = t2 - use;
      const double next = path[s - 1].tend;
      const bool cut = t1 <= next;
      if (t1 <= next) { t1 = next; if (next > t0) sw = true; else more = false; }
      sig_mix(sig, ((uint64_t)s << 16) | ((uint64_t)ndbl << 6) | ((uint64_t)order << 1) | (cut ? 1u : 0u));
      const int base = order - 2;
      for (int k = base + order - 1; k >= base; --k) {
        const double tp = 0.5 * ((t2 - t1) * G.loc[k] + (t2 + t1));
        const double tau = t - tp;
        const double ct = 12.0 * P.a * tau;
        Loc L = beam_loc(P, path, tp, s);
        const double qb = L.q * beta;
        const double dtau = 0.5 * (t2 - t1) * G.w[k];
        const bool keep = qb > 0.0 && dtau > 0.0;
        sig_mix(sig, keep ? 3u : 2u);
        if (keep) add_node(N, L.x, L.y, L.z, B.ax * B.ax + ct, B.ay * B.ay + ct, B.az * B.az + ct, dtau, qb);
      }
      if (sw) --s;
      tpp += (t2 - t1);
      t2 = t1;
      if (tpp >= 2 * stepmax - step0) { stepmax *= 2.0; ++ndbl; if (order != 2) order /= 2; }
    }
  }
}

// Path compression (GaussCompressIntegrate, src/Calc.cpp:213-501): the backward walk of
// gauss_nodes, except that where an interval would reach into the previous segment, the
// segments whose end points lie within the heat's diffusion distance r of the beam position
// at t2 (r^2 = ln2/8 ax^2 (12 a (t - t2) / ax^2 + 1)) and whose power matches are combined
// into one interval, integrated with the Gauss nodes of one point: the power-and-time
// weighted centre of the combined stretch and its mean power.  Restated as the reference
// computes it, including:
//  - the node power is multiplied by beta once per node inside the node loop, so the k-th
//    node of a combined interval carries beta^(k+1) (src/Calc.cpp:453-464);
//  - the combined node's z is never set by the reference (an uninitialised int_seg,
//    src/Calc.cpp:433); its builds give 0 on paths at z = 0.  Here it is the z of the
//    segment the interval starts from;
//  - a segment end outside the r_max box makes the reference's skip loop spin forever
//    (src/Calc.cpp:303-316 never moves to another segment); here the walk stops and the
//    node list is flagged (P.walk_error).
void gauss_compress_nodes(const Problem& P, double t, bool is_sol, Nodes& N) {
  const GaussTables& G = gauss();
  for (size_t b = 0; b < P.paths.size(); ++b) {
    const Beam& B = P.beams[b];
    const std::vector<Seg>& path = P.paths[b];
    int s = find_seg(path, t);
    const double beta = std::pow(3.0 / kPi, 1.5) * B.q / (P.rho * P.cps);
    const double t0 = 0.0;
    double step0 = B.nond;
    if (is_sol) step0 *= B.az;
    double stepmax = step0;
    int order = 16;
    {
      Loc L = beam_loc(P, path, t, s);
      const double qb = L.q * beta;
      if (t <= path.back().tend && qb > 0.0)
        add_node(N, L.x, L.y, L.z, B.ax * B.ax + 0.0, B.ay * B.ay + 0.0, B.az * B.az + 0.0, 0.0, qb);
    }
    double t2 = t, t1 = t, tpp = 0.0;
    if (t > path.back().tend) { tpp += t - path.back().tend; t2 = path.back().tend; }
    while (tpp >= 2 * stepmax - step0) { stepmax *= 2.0; if (order != 2) order /= 2; }
    bool more = true;
    while (more) {
      double sum_t = 0, sum_qt = 0, sum_qtx = 0, sum_qty = 0;
      int s2, ncomb = 0;
      // segment ends outside the r_max box are skipped (src/Calc.cpp:303-316)
      {
        const double ts = path[s].tend;
        if (ts <= t0) break;
        if (!in_rmax(P, path[s].x, path[s].y)) { P.walk_error = true; break; }
      }
      while (tpp >= 2 * stepmax - step0) { stepmax *= 2.0; if (order != 2) order /= 2; }
      const double rt = ref_time(path, B, tpp, s);
      const double use = (rt < stepmax) ? rt : stepmax;
      const Loc Lp = beam_loc(P, path, t2, s);
      const double xp = Lp.x, yp = Lp.y;
      const double r2 = std::log(2.0) / 8.0 * (B.ax * B.ax) * (12.0 * (t - t2) * P.a / (B.ax * B.ax) + 1.0);
      s2 = s;
      t1 = path[s - 1].tend;
      if (t1 < t2 - use) {
        t1 = t2 - use;
      } else {
        while (true) {                                   // combine segments (src/Calc.cpp:350-425)
          if (path[s2 - 1].tend <= t0) { more = false; break; }
          double xs = path[s2 - 1].x, ys = path[s2 - 1].y;
          const double dist2 = (xs - xp) * (xs - xp) + (ys - yp) * (ys - yp);
          const double ts = path[s2 - 1].tend;
          if (!in_rmax(P, xp, yp)) break;
          bool stop = false;
          if ((dist2 > r2) || (path[s2].q != path[s2 - 1].q && (order > 2 || (t2 - ts) > (stepmax / 64.0)))) {
            if (path[s2].mode) {
              sum_qtx += path[s2].x * path[s2].q * (t1 - ts);
              sum_qty += path[s2].y * path[s2].q * (t1 - ts);
              sum_qt += path[s2].q * (t1 - ts);
              sum_t += (t1 - ts);
              t1 = ts;
            } else {
              const double dx = path[s2].x - path[s2 - 1].x, dy = path[s2].y - path[s2 - 1].y;
              const double dt = path[s2].tend - ts;
              double t_int = ts + dt * (std::sqrt(((xp - xs) * (xp - xs) + (yp - ys) * (yp - ys)) / (dx * dx + dy * dy)) -
                                        std::sqrt(r2 / (dx * dx + dy * dy)));
              if (t_int < t2 - stepmax) t_int = t2 - stepmax;
              sum_qtx += (xs + dx * ((t1 + t_int) / 2.0 - ts) / dt) * path[s2].q * (t1 - t_int);
              sum_qty += (ys + dy * ((t1 + t_int) / 2.0 - ts) / dt) * path[s2].q * (t1 - t_int);
              sum_qt += path[s2].q * (t1 - t_int);
              sum_t += (t1 - t_int);
              t1 = t_int;
            }
            stop = true;
          } else {
            if (ts < t2 - stepmax) { stop = true; t1 = t2 - stepmax; }
            else { t1 = ts; ncomb++; }
            const double dt = path[s2].tend - t1;
            if (path[s2].mode) {
              sum_qtx += path[s2].x * path[s2].q * dt;
              sum_qty += path[s2].y * path[s2].q * dt;
              sum_qt += path[s2].q * dt;
              sum_t += dt;
            } else {
              const double dx = path[s2].x - path[s2 - 1].x, dy = path[s2].y - path[s2 - 1].y;
              sum_qtx += (xs + dx * ((path[s2].tend + t1) / 2.0 - ts) / dt) * path[s2].q * dt;
              sum_qty += (ys + dy * ((path[s2].tend + t1) / 2.0 - ts) / dt) * path[s2].q * dt;
              sum_qt += path[s2].q * dt;
              sum_t += dt;
            }
          }
          if (t1 == path[s2 - 1].tend) {
            xs = path[s2 - 1].x;
            ys = path[s2 - 1].y;
            s2--;
            if (!in_rmax(P, xs, ys)) break;
          }
          if (stop) break;
        }
        if (!ncomb) { t1 = path[s - 1].tend; s2 = s - 1; }
      }
      const int base = order - 2;
      if (ncomb) {
        if (sum_qt > 0.0) {
          const double cx = sum_qtx / sum_qt, cy = sum_qty / sum_qt, cz = path[s].z;
          double q = sum_qt / sum_t;
          for (int k = base + order - 1; k >= base; --k) {
            const double tp = 0.5 * ((t2 - t1) * G.loc[k] + (t2 + t1));
            const double ct = 12.0 * P.a * (t - tp);
            q *= beta;
            const double dtau = 0.5 * (t2 - t1) * G.w[k];
            if ((q > 0.0) && (dtau > 0.0))
              add_node(N, cx, cy, cz, B.ax * B.ax + ct, B.ay * B.ay + ct, B.az * B.az + ct, dtau, q);
          }
        }
      } else {
        for (int k = base + order - 1; k >= base; --k) {
          const double tp = 0.5 * ((t2 - t1) * G.loc[k] + (t2 + t1));
          const double ct = 12.0 * P.a * (t - tp);
          Loc L = beam_loc(P, path, tp, s);
          const double qb = L.q * beta;
          const double dtau = 0.5 * (t2 - t1) * G.w[k];
          if (qb > 0.0 && dtau > 0.0)
            add_node(N, L.x, L.y, L.z, B.ax * B.ax + ct, B.ay * B.ay + ct, B.az * B.az + ct, dtau, qb);
        }
      }
      tpp += t2 - t1;
      t2 = t1;
      if (tpp >= 2 * stepmax - step0) { stepmax *= 2.0; if (order != 2) order /= 2; }
      s = s2;
      if (t1 <= t0) more = false;
    }
  }
}

// Method-of-images copies of the node list (src/Calc.cpp:503-608).
void add_bcs(const Problem& P, Nodes& N) {
  std::vector<std::array<int, 3>> all{{0, 0, 0}}, frontier{{0, 0, 0}};
  const double x0 = P.bcx0, x1 = P.bcx1, y0 = P.bcy0, y1 = P.bcy1, z0 = P.bcz0, z1 = P.zmax;
  const int strength = (P.bc_refl != INT_MAX) ? P.bc_refl : 0;
  auto seen = [&](const std::array<int, 3>& c) { return std::find(all.begin(), all.end(), c) != all.end(); };
  for (int it = 0; !frontier.empty() && it < strength; ++it) {
    std::vector<std::array<int, 3>> fresh;
    for (const auto& c0 : frontier) {
      std::array<int, 3> c;
      if (x0 != DBL_MAX) { c = c0; c[0] = -1 - c[0]; if (!seen(c)) { all.push_back(c); fresh.push_back(c); } }
      if (x1 != DBL_MAX) { c = c0; c[0] = 1 - c[0]; if (!seen(c)) { all.push_back(c); fresh.push_back(c); } }
      if (y0 != DBL_MAX) { c = c0; c[1] = -1 - c[1]; if (!seen(c)) { all.push_back(c); fresh.push_back(c); } }
      if (y1 != DBL_MAX) { c = c0; c[1] = 1 - c[1]; if (!seen(c)) { all.push_back(c); fresh.push_back(c); } }
      if (z0 != DBL_MAX) { c = c0; c[2] = -1 - c[2]; if (!seen(c)) { all.push_back(c); fresh.push_back(c); } }
      if (z1 != DBL_MAX) { c = c0; c[2] = 1 - c[2]; if (!seen(c) && c[2] != 1) { all.push_back(c); fresh.push_back(c); } }
    }
    frontier = fresh;
  }
  Nodes src = N;
  N.clear();
  for (const auto& c : all) {
    const int nX = std::abs(c[0] % 2), nY = std::abs(c[1] % 2), nZ = std::abs(c[2] % 2);
    for (size_t i = 0; i < src.size(); ++i) {
      N.xb.push_back((c[0] + nX) * x1 - (c[0] - nX) * x0 + (1 - 2 * nX) * src.xb[i]);
      N.yb.push_back((c[1] + nY) * y1 - (c[1] - nY) * y0 + (1 - 2 * nY) * src.yb[i]);
      N.zb.push_back((c[2] + nZ) * z1 - (c[2] - nZ) * z0 + (1 - 2 * nZ) * src.zb[i]);
      N.ipx.push_back(src.ipx[i]); N.ipy.push_back(src.ipy[i]); N.ipz.push_back(src.ipz[i]);
      N.dtau.push_back(src.dtau[i]); N.expmod.push_back(src.expmod[i]);
    }
  }
}

void make_nodes(const Problem& P, double t, bool is_sol, Nodes& N) {        // src/Calc.cpp:48-65
  N.clear();
  if (P.compress) {
    gauss_compress_nodes(P, t, is_sol, N);
    if (!is_sol) {                         // the smaller of the two lists (the plain one on a tie)
      Nodes R;
      gauss_nodes(P, t, is_sol, R);
      if (R.size() <= N.size()) N = R;
    }
  } else {
    gauss_nodes(P, t, is_sol, N);
  }
  if (P.use_bcs) add_bcs(P, N);
}

// ------------------------------------------------------------------ point sums
inline int pi_(const Problem& P, long p) { return (int)(p / ((long)P.ny * P.nz)); }
inline int pj_(const Problem& P, long p) { return (int)((p / P.nz) % P.ny); }
inline int pk_(const Problem& P, long p) { return (int)(p % P.nz); }
inline long pid(const Problem& P, int i, int j, int k) { return (long)i * ((long)P.nz * P.ny) + (long)j * P.nz + k; }

// Point coordinates from indices (src/Grid.h:310-327); the grid keeps uint16_t counts.
// Custom points keep their own coordinates.
inline double px_(const Problem& P, long p) {
  if (P.custom) return P.cx[p];
  return (P.gx - 1) ? P.xmin + (double(pi_(P, p)) * ((P.xmax - P.xmin) / (P.gx - 1))) : P.xmax;
}
inline double py_(const Problem& P, long p) {
  if (P.custom) return P.cy[p];
  return (P.gy - 1) ? P.ymin + (double(pj_(P, p)) * ((P.ymax - P.ymin) / (P.gy - 1))) : P.ymax;
}
inline double pz_(const Problem& P, long p) {
  if (P.custom) return P.cz[p];
  return (P.gz - 1) ? P.zmin + (double(pk_(P, p)) * ((P.zmax - P.zmin) / (P.gz - 1))) : P.zmax;
}

double sum_T(Problem& P, const Nodes& N, long p) {                           // src/Grid.cpp:281-298
  const double xp = px_(P, p), yp = py_(P, p), zp = pz_(P, p);
  double dT = 0;
  for (size_t n = 0; n < N.size(); ++n) {
    const double dx = xp - N.xb[n], dy = yp - N.yb[n], dz = zp - N.zb[n];
    const double phi = std::exp(-3.0 * ((dx * dx * N.ipx[n]) + (dy * dy * N.ipy[n]) + (dz * dz * N.ipz[n])) + N.expmod[n]);
    dT += N.dtau[n] * phi;
  }
  P.pairs.fetch_add((long long)N.size(), std::memory_order_relaxed);
  return P.T0 + dT;
}

// Calc_T with set = true (src/Grid.cpp:300-311).
double eval_set(Problem& P, const Nodes& N, long p) {
  const double T = sum_T(P, N, p);
  P.T[p] = T;
  if (!P.band.empty()) P.band[p] = std::min(P.band[p], std::fabs(T - P.TL));
  if (!P.calc.empty()) P.calc[p] = 1;
  if (T >= P.TL) {
    if (!P.G.empty()) P.G[p] = DBL_MIN;
    if (!P.V.empty()) P.V[p] = DBL_MIN;
    if (!P.eqFrac.empty()) P.eqFrac[p] = -1.0;
    if (!P.outflag.empty()) P.outflag[p] = 1;
  }
  return T;
}

// C int abs() applied to a double (the reference's unqualified abs on doubles resolves to
// int abs(int), src/Grid.cpp:381,535).  Out-of-range values take the x86-64 conversion
// result INT_MIN, whose abs() stays INT_MIN.
inline double int_abs(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return -2147483648.0;
  const int i = (int)x;
  if (i == INT_MIN) return -2147483648.0;
  return (double)(i < 0 ? -i : i);
}

void solid_fields(Problem& P, long p, double tsol, double* out);

void solidify(Problem& P, double t, long p) {                                 // src/Grid.cpp:316-338
  P.numMelt[p] += 1;
  if (!P.do_sol) return;
  // secant search for the liquidus crossing (src/Grid.cpp:340-404)
  double T2 = P.T[p], T1 = P.T_last[p];
  P.sol_dT[p] = T2 - T1;
  const double T0 = P.TL;
  double t2 = t, t1 = t - P.dt, tsol = 0.0;
  Nodes N;
  for (int it = 1;; ++it) {
    const double m = (T2 - T1) / (t2 - t1);
    tsol = t1 + ((T0 - T1) / m);
    make_nodes(P, tsol, false, N);
    const double Tt = sum_T(P, N, p);
    const double err = int_abs(1.0 - Tt / T0);
    if ((err < P.sol_tol) || (it >= P.sol_iter)) break;
    if (Tt > T0) { t1 = tsol; T1 = Tt; } else { t2 = tsol; T2 = Tt; }
  }
  P.tSol[p] = tsol;
  if (P.o_rdf) { P.rdf_tl[p].push_back(tsol); P.rdf_dT[p].push_back(P.sol_dT[p]); }
  double out[10];
  solid_fields(P, p, tsol, out);
  if (P.o_rdf) P.rdf_cr[p].push_back(out[4]);
  P.G[p] = out[0]; P.Gx[p] = out[1]; P.Gy[p] = out[2]; P.Gz[p] = out[3];
  P.dTdt[p] = out[4]; P.V[p] = out[5]; P.eqFrac[p] = out[6];
}

// Nodes at tsol with the refined schedule, then the gradient / Laplacian / source sums
// (src/Grid.cpp:406-453) and the derived fields (src/Grid.cpp:522-548):
// out = {G, Gx/G, Gy/G, Gz/G, dTdt, V, eqFrac}, then three numbers that say how well the
// fields are conditioned: the cooling rate before its integer truncation, a * lap + dT_t,
// the magnitude its terms add up to, a * sum |seg (dp^2 + dd)| + sum |dT_t terms|, and the
// magnitude of the gradient's terms, sum |seg| |dp| (out[7..9]).
void solid_fields(Problem& P, long p, double tsol, double* out) {
  Nodes N;
  make_nodes(P, tsol, true, N);
  const double xp = px_(P, p), yp = py_(P, p), zp = pz_(P, p);
  double gx = 0, gy = 0, gz = 0, lap = 0, dTt = 0, lap_mag = 0, dtt_mag = 0, g_mag = 0;
  for (size_t n = 0; n < N.size(); ++n) {
    const double dx = xp - N.xb[n], dy = yp - N.yb[n], dz = zp - N.zb[n];
    const double phi = std::exp(-3.0 * ((dx * dx * N.ipx[n]) + (dy * dy * N.ipy[n]) + (dz * dz * N.ipz[n])) + N.expmod[n]);
    const double seg = N.dtau[n] * phi;
    const double ddx = (-6.0 * N.ipx[n]), ddy = (-6.0 * N.ipy[n]), ddz = (-6.0 * N.ipz[n]);
    const double dpx = ddx * dx, dpy = ddy * dy, dpz = ddz * dz;
    gx += seg * dpx; gy += seg * dpy; gz += seg * dpz;
    lap += seg * (dpx * dpx + dpy * dpy + dpz * dpz + ddx + ddy + ddz);
    dTt += (N.dtau[n] == 0) ? phi : 0;
    lap_mag += std::fabs(seg) * (dpx * dpx + dpy * dpy + dpz * dpz - (ddx + ddy + ddz));
    dtt_mag += (N.dtau[n] == 0) ? std::fabs(phi) : 0;
    g_mag += std::fabs(seg) * std::sqrt(dpx * dpx + dpy * dpy + dpz * dpz);
  }
  P.pairs.fetch_add((long long)N.size(), std::memory_order_relaxed);
  // derived quantities (src/Grid.cpp:522-548)
  const double G = std::sqrt(gx * gx + gy * gy + gz * gz);
  const double dTdt = int_abs(P.a * lap + dTt);
  const double V = dTdt / G;
  const double eq = (1.0 - std::exp((-4 * kPi * P.cetN0 / 3) * std::pow(G * (P.cetn + 1) / (std::pow(P.ceta * V, 1 / P.cetn)), -3)));
  out[0] = G; out[1] = gx / G; out[2] = gy / G; out[3] = gz / G; out[4] = dTdt; out[5] = V; out[6] = eq;
  out[7] = P.a * lap + dTt; out[8] = P.a * lap_mag + dtt_mag; out[9] = g_mag;
}

// ------------------------------------------------------------------ melt tracking
// Seed points along the path between t_start and t_end (src/Melt.cpp:20-183).
void beam_trace(Problem& P, double t_start, double t_end, std::vector<long>& out) {
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  auto claim = [&](long p) { if (!P.calc[p]) { out.push_back(p); P.calc[p] = 1; } };
  for (size_t b = 0; b < P.paths.size(); ++b) {               // perimeter points
    const std::vector<Seg>& path = P.paths[b];
    const Beam& B = P.beams[b];
    const double tsub = (P.rcheck * P.rcheck - 1) * (B.ax * B.ax) / (12.0 * P.a);
    const double ts = (t_end - tsub < 0.0) ? 0.0 : t_end - tsub;
    const double te = t_end;
    const double r2 = P.rcheck * P.rcheck * B.ax * B.ax;
    auto perim = [&](int fixed, bool xfixed, int lo, int hi, double x, double y) {
      for (int v = lo; v < hi; ++v) {
        const int i = xfixed ? fixed : v, j = xfixed ? v : fixed;
        const double xp = P.xmin + i * P.xres, yp = P.ymin + j * P.yres;
        const double dx = xp - x, dy = yp - y;
        if (dx * dx + dy * dy < r2) claim(pid(P, i, j, nz - 1));
      }
    };
    auto edges = [&](double x, double y) {
      const int xg = (int)std::floor((x - P.xmin) / P.xres), yg = (int)std::floor((y - P.ymin) / P.yres);
      if (xg < 0) perim(0, true, 0, ny, x, y);
      if (xg > nx - 1) perim(nx - 1, true, 0, ny, x, y);
      if (yg < 0) perim(0, false, 0, nx, x, y);
      if (yg > ny - 1) perim(ny - 1, false, 0, nx, x, y);
    };
    int s0 = 0; while (path[s0].tend < ts && (s0 + 1) != (int)path.size()) ++s0;
    int s1 = 0; while (path[s1].tend < te && (s1 + 1) != (int)path.size()) ++s1;
    for (int s = std::max(s0 - 1, 0); s <= s1; ++s) edges(path[s].x, path[s].y);
    if (path[s1].mode == 0 && te < path.back().tend) { Loc L = beam_loc(P, path, te, s1); edges(L.x, L.y); }
  }
  for (size_t b = 0; b < P.paths.size(); ++b) {               // points under the path
    const std::vector<Seg>& path = P.paths[b];
    auto cell = [&](double x, double y) {
      const int xg = (int)std::floor((x - P.xmin) / P.xres), yg = (int)std::floor((y - P.ymin) / P.yres);
      if (xg < 0 || xg > nx - 1 || yg < 0 || yg > ny - 1) return;
      for (int dx = 0; dx <= 1; ++dx) for (int dy = 0; dy <= 1; ++dy) {
        const int i = xg + dx, j = yg + dy;
        if (i < 0 || i > nx - 1 || j < 0 || j > ny - 1) continue;
        claim(pid(P, i, j, nz - 1));
      }
    };
    int s0 = 0; while (path[s0].tend < t_start && (s0 + 1) != (int)path.size()) ++s0;
    int s1 = 0; while (path[s1].tend < t_end && (s1 + 1) != (int)path.size()) ++s1;
    for (int s = std::max(s0 - 1, 0); s <= s1; ++s) cell(path[s].x, path[s].y);
    if (path[s1].mode == 0 && t_end < path.back().tend) { Loc L = beam_loc(P, path, t_end, s1); cell(L.x, L.y); }
  }
}

template <class F> void par_for(long n, int threads, F f) {
  #pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
  for (long i = 0; i < n; ++i) f(i);
}

// Evaluate T (set) at the given points; returns which are liquid.
void eval_list(Problem& P, const Nodes& N, const std::vector<long>& pts, std::vector<long>& liquid, int threads) {
  std::vector<unsigned char> liq(pts.size());
  par_for((long)pts.size(), threads, [&](long i) { liq[i] = eval_set(P, N, pts[i]) >= P.TL; });
  for (size_t i = 0; i < pts.size(); ++i) if (liq[i]) liquid.push_back(pts[i]);
}

// One frontier-expansion round (src/Melt.cpp:185-269).
void neighbor_round(Problem& P, const Nodes& N, std::vector<long>& test, std::vector<long>& liq,
                    std::vector<long>& reset, bool surface, int threads) {
  std::vector<long> cand;
  for (long p : test) {
    const int i = pi_(P, p), j = pj_(P, p), k = pk_(P, p);
    for (int di = -1; di <= 1; ++di) for (int dj = -1; dj <= 1; ++dj) {
      const int ni = i + di, nj = j + dj;
      if (ni < 0 || ni > P.nx - 1 || nj < 0 || nj > P.ny - 1) continue;
      if (surface) {
        const long q = pid(P, ni, nj, k);
        if (!P.calc[q]) { P.calc[q] = 1; cand.push_back(q); }
      } else {
        for (int dk = -1; dk < 1; ++dk) {
          const int nk = k + dk;
          if (nk < 0) continue;
          const long q = pid(P, ni, nj, nk);
          if (!P.calc[q]) { P.calc[q] = 1; cand.push_back(q); }
        }
      }
    }
  }
  std::vector<long> hot;
  eval_list(P, N, cand, hot, threads);
  liq.insert(liq.end(), hot.begin(), hot.end());
  reset.insert(reset.end(), cand.begin(), cand.end());
  test.swap(hot);
}

void alloc_state(Problem& P) {
  const long n = P.pnum;
  P.T.assign(n, 0.0);
  if (P.mode == 1 || P.tracking != TRACK_NONE) { P.calc.assign(n, 0); P.outflag.assign(n, 0); P.band.assign(n, DBL_MAX); }
  if (P.mode == 1) {
    P.T_last.assign(n, 0.0);
    P.tSol.assign(n, 0.0); P.G.assign(n, 0.0); P.V.assign(n, 0.0); P.Gx.assign(n, 0.0); P.Gy.assign(n, 0.0);
    P.Gz.assign(n, 0.0); P.dTdt.assign(n, 0.0); P.eqFrac.assign(n, 0.0); P.depth.assign(n, 0.0);
    P.numMelt.assign(n, 0);
    P.sol_dT.assign(n, 0.0);
    if (P.o_rdf) { P.rdf_tm.assign(n, {}); P.rdf_tl.assign(n, {}); P.rdf_cr.assign(n, {}); P.rdf_dT.assign(n, {}); }
  }
}

bool finished(const Problem& P, double t, long liq) { return t > P.end_time && liq == 0; }   // src/Util.cpp:239-243

// src/Run.cpp:409-467
int64_t run_notracking(Problem& P, int threads, int64_t max_steps, double budget_s) {
  const double t_start = omp_get_wtime();
  std::fill(P.T.begin(), P.T.end(), P.T0);
  Nodes N;
  double t = 0.0;
  int64_t step = 0;
  while (true) {
    make_nodes(P, t, false, N);
    P.T_last = P.T;
    long liq = 0;
    #pragma omp parallel for num_threads(threads) schedule(dynamic, 256) reduction(+:liq)
    for (long p = 0; p < P.pnum; ++p) {
      if (!(eval_set(P, N, p) >= P.TL)) { if (P.T_last[p] >= P.TL) solidify(P, t, p); }
      else liq++;
    }
    if (finished(P, t, liq)) break;
    t += P.dt; ++step;
    if (max_steps > 0 && step >= max_steps) return step;            // steps run
    if (budget_s > 0 && omp_get_wtime() - t_start > budget_s) return step;
  }
  return step + 1;
}

// src/Run.cpp:469-573 (Volume) and 575-709 (Surface)
int64_t run_tracking(Problem& P, int threads, int64_t max_steps, double budget_s) {
  const double t_start = omp_get_wtime();
  const bool surface = P.tracking == TRACK_SURFACE;
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  std::vector<long> liq, reset;
  std::vector<int> depths((size_t)nx * ny, 0);
  std::vector<double> depth_max((size_t)nx * ny, 0.0);
  Nodes N, Nlast;
  double t = 0.0;
  int64_t step = 0;
  while (true) {
    make_nodes(P, t, false, N);
    for (long p : reset) {
      // a point still liquid when its step ended opens a melt event (Surface only; one
      // open event at a time: pushed while as many melting as solidification times)
      if (surface && P.o_rdf && P.T[p] >= P.TL && P.rdf_tm[p].size() == P.rdf_tl[p].size())
        P.rdf_tm[p].push_back(t - P.dt);
      P.T_last[p] = P.T[p]; P.calc[p] = 0;
    }
    std::vector<long> last_liq = liq;
    reset = liq;
    liq.clear();
    // re-test last step's liquid points; solidify those that cooled
    {
      const long n = (long)last_liq.size();
      std::vector<unsigned char> still(n);
      std::vector<std::vector<long>> cols(n);
      #pragma omp parallel for num_threads(threads) schedule(dynamic, 4)
      for (long it = 0; it < n; ++it) {
        const long p = last_liq[it];
        if (!(eval_set(P, N, p) >= P.TL)) {
          solidify(P, t, p);
          if (surface) {                                          // solidify the column below
            const int i = pi_(P, p), j = pj_(P, p);
            const size_t dn = (size_t)i * ny + j;
            const int dep = depths[dn];
            for (int d = dep; d > 0; --d) {
              const long q = pid(P, i, j, nz - 1 - d);
              eval_set(P, N, q);
              if (d != dep) P.T_last[q] = sum_T(P, Nlast, q);
              solidify(P, t, q);
              cols[it].push_back(q);
            }
            depths[dn] = 0;
          }
        } else still[it] = 1;
      }
      for (long it = 0; it < n; ++it) {
        if (still[it]) liq.push_back(last_liq[it]);
        reset.insert(reset.end(), cols[it].begin(), cols[it].end());
      }
    }
    std::vector<long> test = surface ? last_liq : liq;
    if (step && t < P.end_time + P.dt) {
      std::vector<long> seeds;
      beam_trace(P, t - P.dt, t, seeds);
      reset.insert(reset.end(), seeds.begin(), seeds.end());
      std::vector<long> hot;
      eval_list(P, N, seeds, hot, threads);
      test.insert(test.end(), hot.begin(), hot.end());
      liq.insert(liq.end(), hot.begin(), hot.end());
    }
    while (!test.empty()) neighbor_round(P, N, test, liq, reset, surface, threads);

    if (surface && nz != 1) {                                  // src/Melt.cpp:271-317
      const long n = (long)liq.size();
      std::vector<std::vector<long>> touched(n);
      #pragma omp parallel for num_threads(threads) schedule(dynamic, 4)
      for (long it = 0; it < n; ++it) {
        const long p = liq[it];
        const int i = pi_(P, p), j = pj_(P, p);
        const size_t dn = (size_t)i * ny + j;
        int d = depths[dn];
        bool none_deeper = true;
        while (true) {
          ++d;
          if (d == nz) break;
          const long q = pid(P, i, j, nz - 1 - d);
          touched[it].push_back(q);
          if (!(eval_set(P, N, q) >= P.TL)) break;
          none_deeper = false;
        }
        while (true) {
          --d;
          if (d == 0 || !none_deeper) break;
          const long q = pid(P, i, j, nz - 1 - d);
          touched[it].push_back(q);
          if (!(eval_set(P, N, q) >= P.TL)) {
            if (d != depths[dn]) P.T_last[q] = sum_T(P, Nlast, q);
            solidify(P, t, q);
          } else break;
        }
        if (d == nz) --d;
        depths[dn] = d;
      }
      for (long it = 0; it < n; ++it) reset.insert(reset.end(), touched[it].begin(), touched[it].end());
    }
    if (surface && nz != 1 && P.o_depth) {                     // src/Melt.cpp:319-357
      for (long p : liq) {
        const int i = pi_(P, p), j = pj_(P, p);
        const size_t dn = (size_t)i * ny + j;
        const int dl = depths[dn];
        double dep;
        if (dl == nz - 1) dep = dl;
        else {
          const double Tl = P.T[pid(P, i, j, nz - 1 - dl)], Ts = P.T[pid(P, i, j, nz - 1 - (dl + 1))];
          dep = dl + (P.TL - Tl) / (Ts - Tl);
        }
        if (dep > depth_max[dn]) {
          depth_max[dn] = dep;
          for (int d = dl; d >= 0; --d) P.depth[pid(P, i, j, nz - 1 - d)] = dep;
        }
      }
    }
    if (finished(P, t, (long)liq.size())) break;
    t += P.dt; ++step;
    Nlast = N;
    if (max_steps > 0 && step >= max_steps) return step;            // steps run
    if (budget_s > 0 && omp_get_wtime() - t_start > budget_s) return step;
  }
  return step + 1;
}

// Run::Stork (src/Run.cpp:711-1079): the Surface loop's frontier expansion over the top
// layer, without solidification, then per liquid column a walk that finds its depth and
// marks its layers liquid; every cell (8 grid points) whose count of liquid points changed
// or is neither 0 nor 8 at this or the previous step gets a row: its index, the two step
// times and the temperatures of its points at both.
int64_t run_stork(Problem& P, int threads, int64_t max_steps, double budget_s) {
  const double t_start = omp_get_wtime();
  const int nx = P.nx, ny = P.ny, nz = P.nz;
  const int cx = nx - 1, cy = ny - 1, cz = nz - 1;
  const long cpnum = (long)cx * cy * cz;
  std::vector<uint8_t> c_a(std::max(cpnum, 0L), 0), c_b(std::max(cpnum, 0L), 0);
  std::vector<double> T_a(P.pnum, P.T0), T_b(P.pnum, P.T0);
  std::vector<uint8_t> calc_a(P.pnum, 1), calc_b(P.pnum, 1), is_liq(P.pnum, 0);
  std::vector<long> liq, reset;
  std::vector<int> depths((size_t)nx * ny, 0);
  Nodes N, Nlast;
  double t = 0.0;
  int64_t itert = 0;
  while (true) {
    std::vector<uint8_t>& c_prev = (itert % 2) ? c_a : c_b;
    std::vector<uint8_t>& c_cur = (itert % 2) ? c_b : c_a;
    std::vector<double>& T_prev = (itert % 2) ? T_a : T_b;
    std::vector<double>& T_cur = (itert % 2) ? T_b : T_a;
    std::vector<uint8_t>& calc_prev = (itert % 2) ? calc_a : calc_b;
    std::vector<uint8_t>& calc_cur = (itert % 2) ? calc_b : calc_a;
    std::fill(c_cur.begin(), c_cur.end(), 0);
    std::fill(calc_cur.begin(), calc_cur.end(), 0);
    std::fill(is_liq.begin(), is_liq.end(), 0);
    for (long p : reset) { P.T_last[p] = P.T[p]; P.calc[p] = 0; }
    reset.clear();
    const std::vector<long> last_liq = liq;
    liq.clear();
    make_nodes(P, t, false, N);
    for (long p : last_liq) {                                   // re-test last step's liquid points
      T_cur[p] = eval_set(P, N, p);
      calc_cur[p] = 1;
      reset.push_back(p);
      if (T_cur[p] >= P.TL) liq.push_back(p);
      else depths[(size_t)pi_(P, p) * ny + pj_(P, p)] = 0;
    }
    std::vector<long> test = liq;
    if (itert && t < P.end_time + P.dt) {
      std::vector<long> seeds;
      beam_trace(P, t - P.dt, t, seeds);
      for (long p : seeds) {
        reset.push_back(p);
        if (calc_cur[p] == 0) {
          T_cur[p] = eval_set(P, N, p);
          calc_cur[p] = 1;
          if (T_cur[p] >= P.TL) { test.push_back(p); liq.push_back(p); }
        }
      }
    }
    while (!test.empty()) {                                     // frontier expansion, top layer
      std::vector<long> next;
      for (long p : test) {
        const int i = pi_(P, p), j = pj_(P, p), k = pk_(P, p);
        for (int di = 0; di < 3; ++di) for (int dj = 0; dj < 3; ++dj) {
          const int ni = i + di - 1, nj = j + dj - 1;
          if (ni < 0 || ni > nx - 1 || nj < 0 || nj > ny - 1) continue;
          const long q = pid(P, ni, nj, k);
          if (P.calc[q]) continue;
          T_cur[q] = eval_set(P, N, q);
          calc_cur[q] = 1;
          if (T_cur[q] >= P.TL) { liq.push_back(q); next.push_back(q); }
          reset.push_back(q);
        }
      }
      test.swap(next);
    }
    for (long p : liq) {                                        // depths (src/Run.cpp:909-956)
      const int i = pi_(P, p), j = pj_(P, p);
      const size_t dn = (size_t)i * ny + j;
      int depth = depths[dn];
      bool deeper = false;
      while (true) {
        depth++;
        if (depth == nz) break;
        const long q = pid(P, i, j, nz - 1 - depth);
        T_cur[q] = sum_T(P, N, q);
        calc_cur[q] = 1;
        if (!(T_cur[q] >= P.TL)) break;
        deeper = true;
      }
      while (true) {
        depth--;
        if (depth == 0 || deeper) break;
        const long q = pid(P, i, j, nz - 1 - depth);
        T_cur[q] = sum_T(P, N, q);
        calc_cur[q] = 1;
        if (T_cur[q] >= P.TL) break;
      }
      if (depth == nz - 1) depth--;
      depths[dn] = depth;
      for (int d = 0; d <= depth; ++d) is_liq[pid(P, i, j, nz - 1 - d)] = 1;
    }
    // the cells in index order, split over threads in contiguous chunks whose relevant
    // cells are joined in chunk order (the single-thread order)
    std::vector<long> relevant;
    if (!last_liq.empty() || !liq.empty()) {
      const int nt = std::max(1, threads);
      std::vector<std::vector<long>> part(nt);
      #pragma omp parallel num_threads(nt)
      {
        const int th = omp_get_thread_num(), nth = omp_get_num_threads();
        const long c0 = cpnum * th / nth, c1 = cpnum * (th + 1) / nth;
        for (long c = c0; c < c1; ++c) {
          const int ci = (int)((c / cy) / cz), cj = (int)((c / cz) % cy), ck = (int)(c % cz);
          int n = 0;
          for (int di = 0; di < 2; ++di) for (int dj = 0; dj < 2; ++dj) for (int dk = 0; dk < 2; ++dk)
            n += is_liq[pid(P, ci + di, cj + dj, ck + dk)];
          c_cur[c] = (uint8_t)n;
          if (c_cur[c] != c_prev[c] || c_prev[c] % 8 || c_cur[c] % 8) part[th].push_back(c);
        }
      }
      for (const auto& v : part) relevant.insert(relevant.end(), v.begin(), v.end());
    }
    // vertex temperatures: each point's at both times once (the values do not depend on who
    // computes them), then the rows
    {
      std::vector<long> need;
      for (long c : relevant) {
        const int ci = (int)((c / cy) / cz), cj = (int)((c / cz) % cy), ck = (int)(c % cz);
        for (int di = 0; di < 2; ++di) for (int dj = 0; dj < 2; ++dj) for (int dk = 0; dk < 2; ++dk) {
          const long p = pid(P, ci + di, cj + dj, ck + dk);
          if (calc_prev[p] == 0 || calc_cur[p] == 0) need.push_back(p);
        }
      }
      std::sort(need.begin(), need.end());
      need.erase(std::unique(need.begin(), need.end()), need.end());
      par_for((long)need.size(), threads, [&](long i) {
        const long p = need[i];
        if (calc_prev[p] == 0) T_prev[p] = sum_T(P, Nlast, p);
        if (calc_cur[p] == 0) T_cur[p] = sum_T(P, N, p);
      });
      for (long p : need) { calc_prev[p] = 1; calc_cur[p] = 1; }
    }
    for (long c : relevant) {
      const int ci = (int)((c / cy) / cz), cj = (int)((c / cz) % cy), ck = (int)(c % cz);
      P.rrdf_idx.push_back((uint32_t)ci); P.rrdf_idx.push_back((uint32_t)cj); P.rrdf_idx.push_back((uint32_t)ck);
      P.rrdf_t.push_back(t - P.dt); P.rrdf_t.push_back(t);
      double Ts[16];
      int n = 0;
      for (int di = 0; di < 2; ++di) for (int dj = 0; dj < 2; ++dj) for (int dk = 0; dk < 2; ++dk) {
        const long p = pid(P, ci + di, cj + dj, ck + dk);
        Ts[n] = T_prev[p];
        Ts[n + 8] = T_cur[p];
        ++n;
      }
      P.rrdf_T.insert(P.rrdf_T.end(), Ts, Ts + 16);
    }
    if (finished(P, t, (long)liq.size())) break;
    t += P.dt; ++itert;
    Nlast = N;
    if (max_steps > 0 && itert >= max_steps) return itert;
    if (budget_s > 0 && omp_get_wtime() - t_start > budget_s) return itert;
  }
  return itert + 1;
}

}  // namespace

// ====================================================================== C API
extern "C" {

void* or_load(const char* param_input, char* err, int errlen) {
  Problem* P = new Problem();
  std::string e;
  bool ok = false;
  try { ok = load_problem(*P, param_input, e); } catch (const std::exception& ex) { e = ex.what(); ok = false; }
  if (!ok) {
    if (err && errlen > 0) { std::snprintf(err, errlen, "%s", e.c_str()); }
    delete P;
    return nullptr;
  }
  alloc_state(*P);
  return P;
}

void or_free(void* h) { delete (Problem*)h; }

void or_info(void* h, double* info) {
  Problem& P = *(Problem*)h;
  const double v[16] = {(double)P.nx, (double)P.ny, (double)P.nz, (double)P.pnum, (double)P.beams.size(),
                        (double)P.snaps.size(), (double)P.mode, (double)P.tracking, P.dt, P.end_time,
                        P.T0, P.TL, P.r_max, P.a, (double)P.thnum, (double)P.use_bcs};
  std::memcpy(info, v, sizeof(v));
}

double or_snapshot_time(void* h, int idx) { return ((Problem*)h)->snaps.at(idx); }

int or_nodes(void* h, double t, int is_sol, double* out, int cap) {
  Problem& P = *(Problem*)h;
  Nodes N;
  make_nodes(P, t, is_sol != 0, N);
  const int n = (int)N.size(), m = std::min(n, cap);
  const std::vector<double>* f[8] = {&N.xb, &N.yb, &N.zb, &N.ipx, &N.ipy, &N.ipz, &N.dtau, &N.expmod};
  for (int c = 0; c < 8; ++c) for (int i = 0; i < m; ++i) out[(size_t)c * cap + i] = (*f[c])[i];
  return n;
}

void or_calc_T(void* h, double t, const int64_t* pts, int64_t n, double* T, int threads) {
  Problem& P = *(Problem*)h;
  if (threads <= 0) threads = omp_get_max_threads();
  Nodes N;
  make_nodes(P, t, false, N);
  #pragma omp parallel for num_threads(threads) schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) T[i] = sum_T(P, N, (long)pts[i]);
}

void or_snapshot(void* h, int idx, double* T, int threads) {                   // src/Run.cpp:80-124
  Problem& P = *(Problem*)h;
  if (threads <= 0) threads = omp_get_max_threads();
  Nodes N;
  make_nodes(P, P.snaps.at(idx), false, N);
  #pragma omp parallel for num_threads(threads) schedule(dynamic, 1 + P.pnum / threads / 128)
  for (long p = 0; p < P.pnum; ++p) T[p] = sum_T(P, N, p);
}

int64_t or_solidify_budget(void* h, int threads, int64_t max_steps, double budget_s) {
  Problem& P = *(Problem*)h;
  if (threads <= 0) threads = omp_get_max_threads();
  if (P.mode != 1) return -1;
  if (P.tracking == TRACK_NONE) return run_notracking(P, threads, max_steps, budget_s);
  if (P.tracking == TRACK_STORK) return run_stork(P, threads, max_steps, budget_s);
  return run_tracking(P, threads, max_steps, budget_s);
}

int64_t or_solidify(void* h, int threads, int64_t max_steps) { return or_solidify_budget(h, threads, max_steps, 0.0); }

int or_field(void* h, const char* name, double* out) {
  Problem& P = *(Problem*)h;
  const std::string f(name);
  const std::vector<double>* v = nullptr;
  if (f == "band") v = &P.band; else if (f == "sol_dT") v = &P.sol_dT;
  else if (f == "T") v = &P.T; else if (f == "tSol") v = &P.tSol; else if (f == "G") v = &P.G;
  else if (f == "V") v = &P.V; else if (f == "Gx") v = &P.Gx; else if (f == "Gy") v = &P.Gy;
  else if (f == "Gz") v = &P.Gz; else if (f == "dTdt") v = &P.dTdt; else if (f == "eqFrac") v = &P.eqFrac;
  else if (f == "depth") {
    // get_depth scales the stored fractional depth by the z spacing (src/Grid.h:340-342)
    if (P.depth.empty()) return 1;
    const double dz = (P.zmax - P.zmin) / (P.gz - 1);
    for (long p = 0; p < P.pnum; ++p) out[p] = P.depth[p] * dz;
    return 0;
  }
  if (v) { if (v->empty()) return 1; std::memcpy(out, v->data(), sizeof(double) * P.pnum); return 0; }
  if (f == "numMelt") {
    if (P.numMelt.empty()) return 1;
    // with RDF the count is the number of melting times (src/Grid.h:232,343-350)
    for (long p = 0; p < P.pnum; ++p) out[p] = P.o_rdf ? (double)P.rdf_tm[p].size() : P.numMelt[p];
    return 0;
  }
  if (f == "output_flag") {
    for (long p = 0; p < P.pnum; ++p) out[p] = P.outflag.empty() ? 1.0 : (double)P.outflag[p];
    return 0;
  }
  return 2;
}

int64_t or_pairs(void* h) { return ((Problem*)h)->pairs.load(); }

int64_t or_rdf(void* h, int32_t* counts, double* vals, double* dT, int64_t cap) {
  const Problem& P = *(Problem*)h;
  if (!P.o_rdf) return -1;
  int64_t n = 0, m = 0;
  for (long p = 0; p < P.pnum; ++p) {
    const std::vector<double>* v[3] = {&P.rdf_tm[p], &P.rdf_tl[p], &P.rdf_cr[p]};
    for (int c = 0; c < 3; ++c) {
      if (counts) counts[3 * p + c] = (int32_t)v[c]->size();
      for (double x : *v[c]) { if (vals && n < cap) vals[n] = x; ++n; }
    }
    for (double x : P.rdf_dT[p]) { if (dT && m < cap) dT[m] = x; ++m; }
  }
  return n;
}

int64_t or_rrdf(void* h, uint32_t* idx, double* ts, double* Ts, int64_t cap) {
  const Problem& P = *(Problem*)h;
  const int64_t n = (int64_t)P.rrdf_t.size() / 2;
  for (int64_t r = 0; r < std::min(n, cap); ++r) {
    for (int c = 0; c < 3; ++c) idx[3 * r + c] = P.rrdf_idx[3 * r + c];
    for (int c = 0; c < 2; ++c) ts[2 * r + c] = P.rrdf_t[2 * r + c];
    for (int c = 0; c < 16; ++c) Ts[16 * r + c] = P.rrdf_T[16 * r + c];
  }
  return n;
}

void or_solid_fields(void* h, int64_t p, double tsol, double* out) { solid_fields(*(Problem*)h, (long)p, tsol, out); }

void or_solid_fields_many(void* h, const int64_t* pts, const double* tsol, int64_t n, double* out, int threads) {
  Problem& P = *(Problem*)h;
  if (threads <= 0) threads = omp_get_max_threads();
  #pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) solid_fields(P, (long)pts[i], tsol[i], out + 10 * i);
}

uint64_t or_schedule(void* h, double t, int is_sol) {
  Problem& P = *(Problem*)h;
  Nodes N;
  uint64_t sig = 1469598103934665603ull;
  gauss_nodes(P, t, is_sol != 0, N, &sig);
  sig_mix(&sig, (uint64_t)N.size());
  return sig;
}

void or_schedule_many(void* h, const double* t, int64_t n, int is_sol, uint64_t* out, int threads) {
  if (threads <= 0) threads = omp_get_max_threads();
  #pragma omp parallel for num_threads(threads) schedule(dynamic, 16)
  for (int64_t i = 0; i < n; ++i) out[i] = or_schedule(h, t[i], is_sol);
}

}  // extern "C"
