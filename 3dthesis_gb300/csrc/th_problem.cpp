// Deck reader for the reference's keyword-file inputs and the derived constants.
//
// Semantics follow src/Init.cpp:33-908 and src/Util.cpp:76-166: brace blocks keyed by
// the first token of a line, "key value" pairs one per line, defaults for anything not
// given, '*' wildcards for multi-beam decks, path files in mm with an implicit origin
// spot and segment end times from speed or dwell.  Unlike the reference, a missing or
// malformed required file is an error instead of a silent default or exit(1).
#include "th_problem.h"

#include <algorithm>
#include <cctype>
#include <cfloat>
#include <climits>
#include <cmath>
#include <fstream>
#include <map>
#include <sstream>

namespace {

const double kPi = 3.14159265358979323846;

// A keyword file as blocks of key -> value strings.  Only the blocks and keys asked for
// are retained; a block name counts only as the first token of a line and must be
// followed by "{" (possibly on a later line).
class KeywordFile {
 public:
  bool read(const std::string& path, const std::vector<std::string>& blocks) {
    std::ifstream in(path.c_str());
    if (!in.is_open()) return false;
    std::vector<std::vector<std::string>> lines;
    std::string line;
    while (std::getline(in, line)) {
      std::vector<std::string> toks;
      std::istringstream ss(line);
      std::string t;
      while (ss >> t) toks.push_back(t);
      if (!toks.empty()) lines.push_back(toks);
    }
    size_t li = 0;
    while (li < lines.size()) {
      const std::string head = lines[li][0];
      ++li;
      if (std::find(blocks.begin(), blocks.end(), head) == blocks.end()) continue;
      counts_[head]++;
      if (li >= lines.size()) break;
      const bool open = lines[li][0] == "{";
      ++li;
      if (!open) continue;
      while (li < lines.size()) {
        const std::vector<std::string>& l = lines[li];
        if (l[0] == "}") { ++li; break; }
        // the value is the next token, which may sit on the following line
        if (l.size() >= 2) { vals_[head][l[0]] = l[1]; ++li; }
        else if (li + 1 < lines.size()) { vals_[head][l[0]] = lines[li + 1][0]; li += 2; }
        else { li = lines.size(); }
      }
    }
    return true;
  }
  std::string str(const std::string& b, const std::string& k) const {
    auto bi = vals_.find(b);
    if (bi == vals_.end()) return "";
    auto ki = bi->second.find(k);
    return ki == bi->second.end() ? "" : ki->second;
  }
  double num(const std::string& b, const std::string& k, double def) const {
    const std::string s = str(b, k);
    return s.empty() ? def : std::stod(s);
  }
  int integer(const std::string& b, const std::string& k, int def) const {
    const std::string s = str(b, k);
    return s.empty() ? def : std::stoi(s);
  }
  bool flag(const std::string& b, const std::string& k, bool def) const {
    const std::string s = str(b, k);
    return s.empty() ? def : (std::stoi(s) != 0);
  }
  int count(const std::string& b) const { auto i = counts_.find(b); return i == counts_.end() ? 0 : i->second; }

 private:
  std::map<std::string, std::map<std::string, std::string>> vals_;
  std::map<std::string, int> counts_;
};

std::string join_dir(const std::string& dir, const std::string& f) {
  if (f.empty() || f[0] == '/') return f;
  return dir + "/" + f;
}

bool exists(const std::string& f) { std::ifstream in(f.c_str()); return in.is_open(); }

std::vector<std::string> wildcard(const std::string& pattern) {
  std::vector<std::string> out;
  const size_t star = pattern.find('*');
  if (star == std::string::npos) { out.push_back(pattern); return out; }
  for (int n = 1;; ++n) {
    std::string f = pattern.substr(0, star) + std::to_string(n) + pattern.substr(star + 1);
    if (!exists(f)) break;
    out.push_back(f);
  }
  return out;
}

bool read_path_file(const std::string& file, std::vector<DevSeg>& path, std::string& err) {
  std::ifstream in(file.c_str());
  if (!in.is_open()) { err = "cannot open path file " + file; return false; }
  path.clear();
  DevSeg origin{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1, 0};
  path.push_back(origin);
  std::string line;
  std::getline(in, line);                       // header
  while (true) {
    DevSeg s{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1, 0};
    if (!(in >> s.mode >> s.x >> s.y >> s.z >> s.q >> s.prm)) break;
    s.x *= 1e-3; s.y *= 1e-3; s.z *= 1e-3;
    path.push_back(s);
    if (!std::getline(in, line)) break;         // rest of the record's line is ignored
  }
  if (path.size() < 2) { err = "path file " + file + " has no segments"; return false; }
  for (size_t k = 1; k < path.size(); ++k) {
    // the reference defines only modes 0 and 1 (src/Util.cpp:198-206); a line needs a
    // positive speed and a spot a non-negative dwell for the end times to increase
    if (path[k].mode != 0 && path[k].mode != 1) { err = "path segment mode must be 0 or 1 in " + file; return false; }
    if ((path[k].mode == 0 && !(path[k].prm > 0.0)) || (path[k].mode == 1 && !(path[k].prm >= 0.0))) {
      err = "path segment speed/dwell out of range in " + file; return false;
    }
  }
  for (size_t k = 1; k < path.size(); ++k) {
    if (path[k].mode) path[k].tend = path[k - 1].tend + path[k].prm;
    else {
      const double dx = path[k].x - path[k - 1].x, dy = path[k].y - path[k - 1].y, dz = path[k].z - path[k - 1].z;
      path[k].tend = path[k - 1].tend + std::sqrt(dx * dx + dy * dy + dz * dz) / path[k].prm;
    }
  }
  return true;
}

int parse_tracking(const std::string& s, bool& ok) {
  ok = true;
  if (s.empty() || s == "None") return TH_TRACK_NONE;
  if (s == "Volume") return TH_TRACK_VOLUME;
  if (s == "Surface") return TH_TRACK_SURFACE;
  if (s == "Stork") return TH_TRACK_STORK;
  ok = false;
  return TH_TRACK_NONE;
}

// Axis set-up (src/Init.cpp:866-908); the z branch tests the y count, as the reference does.
void axis(int& num, double& vmin, double& vmax, double& res, bool guard_is_one) {
  if (num == INT_MAX) { num = 1 + int(0.5 + (vmax - vmin) / res); vmax = vmin + (num - 1) * res; }
  else if (!guard_is_one) res = (vmax - vmin) / (num - 1);
  else res = DBL_MAX;
}

// Division by an invariant divisor d >= 1 for dividends x < 2^31 (Granlund and Montgomery,
// "Division by invariant integers using multiplication", 1994): with l = ceil(log2 d),
// s = 31 + l and m = ceil(2^s / d), m < 2^32 and floor(x / d) = floor(x * m / 2^s), because
// the excess x * (m d - 2^s) / (d 2^s) stays below x / 2^s < 1 / d (m d - 2^s < d <= 2^l).
void udiv_magic(uint32_t d, uint32_t& m, int32_t& s) {
  int l = 0;
  while ((1ull << l) < d) ++l;
  s = 31 + l;
  m = (uint32_t)(((1ull << s) + d - 1) / d);
}

}  // namespace

void th_gauss_tables(double loc[30], double w[30]) {
  const int orders[4] = {2, 4, 8, 16};
  for (int oi = 0; oi < 4; ++oi) {
    const int n = orders[oi];
    for (int i = 0; i < n; ++i) {
      // Newton iteration on P_n from the standard cosine guess, roots ascending
      double x = std::cos(kPi * ((n - i) - 0.25) / (n + 0.5));
      double dpn = 1.0;
      for (int it = 0; it < 100; ++it) {
        double pm = 1.0, pn = x;
        for (int k = 2; k <= n; ++k) { const double pk = ((2.0 * k - 1.0) * x * pn - (k - 1.0) * pm) / k; pm = pn; pn = pk; }
        dpn = n * (x * pn - pm) / (x * x - 1.0);
        const double step = pn / dpn;
        x -= step;
        if (std::fabs(step) < 1e-17) break;
      }
      double pm = 1.0, pn = x;
      for (int k = 2; k <= n; ++k) { const double pk = ((2.0 * k - 1.0) * x * pn - (k - 1.0) * pm) / k; pm = pn; pn = pk; }
      dpn = n * (x * pn - pm) / (x * x - 1.0);
      loc[n - 2 + i] = std::round(x * 1e8) / 1e8;
      w[n - 2 + i] = std::round(2.0 / ((1.0 - x * x) * dpn * dpn) * 1e8) / 1e8;
    }
  }
}

bool th_load_deck(const std::string& param_input, HostProblem& hp, std::string& err) {
  try {
    const size_t slash = param_input.find_last_of('/');
    hp.dir = slash == std::string::npos ? "." : param_input.substr(0, slash);
    KeywordFile top;
    if (!top.read(param_input, {"Simulation", "Options"})) { err = "cannot open " + param_input; return false; }
    hp.name = top.str("Simulation", "Name");
    if (hp.name.empty()) hp.name = "N/A";
    const std::string f_mode = top.str("Simulation", "Mode"), f_mat = top.str("Simulation", "Material"),
                      f_beam = top.str("Simulation", "Beam"), f_path = top.str("Simulation", "Path");
    if (f_mode.empty() || f_mat.empty() || f_beam.empty() || f_path.empty()) {
      err = "ParamInput must name the Mode, Material, Beam and Path files"; return false;
    }
    // beams (src/Init.cpp:488-515); q = P * efficiency * 2 (src/Init.cpp:862-865)
    for (const std::string& f : wildcard(join_dir(hp.dir, f_beam))) {
      KeywordFile b;
      if (!b.read(f, {"Shape", "Intensity"})) { err = "cannot open beam file " + f; return false; }
      HostBeam B;
      B.ax = b.num("Shape", "Width_X", 10.0e-6); B.ay = b.num("Shape", "Width_Y", 10.0e-6);
      B.az = b.num("Shape", "Depth_Z", 1.0e-6);
      B.power = b.num("Intensity", "Power", 1200); B.eff = b.num("Intensity", "Efficiency", 1.0);
      if (B.eff == DBL_MAX) B.eff = 1.0;
      B.q = B.power * B.eff * 2.0;
      if (!(B.ax > 0.0 && B.ay > 0.0 && B.az > 0.0)) { err = "beam widths must be positive in " + f; return false; }
      hp.beams.push_back(B);
    }
    if (hp.beams.empty()) { err = "no beam files match " + f_beam; return false; }
    if ((int)hp.beams.size() > TH_MAX_BEAMS) { err = "more than TH_MAX_BEAMS beams"; return false; }
    // material (src/Init.cpp:410-443)
    {
      KeywordFile m;
      if (!m.read(join_dir(hp.dir, f_mat), {"Constants", "CET"})) { err = "cannot open material file"; return false; }
      hp.T0 = m.num("Constants", "T_0", 1273.0); hp.TL = m.num("Constants", "T_L", 1610.0);
      hp.kon = m.num("Constants", "k", 26.6); hp.cps = m.num("Constants", "c", 600.0);
      hp.rho = m.num("Constants", "p", 7451.0);
      hp.cetN0 = m.num("CET", "N0", DBL_MAX); hp.cetn = m.num("CET", "n", DBL_MAX); hp.ceta = m.num("CET", "a", DBL_MAX);
      hp.a = hp.kon / (hp.rho * hp.cps);
    }
    for (HostBeam& B : hp.beams) B.nond = B.ax * B.ax / hp.a;
    // paths
    for (const std::string& f : wildcard(join_dir(hp.dir, f_path))) {
      std::vector<DevSeg> path;
      if (!read_path_file(f, path, err)) return false;
      hp.paths.push_back(path);
    }
    if (hp.paths.size() != hp.beams.size()) { err = "beam and path file counts differ"; return false; }
    hp.end_time = 0.0;
    for (const auto& p : hp.paths) hp.end_time = std::max(hp.end_time, p.back().tend);
    // mode (src/Init.cpp:305-408)
    {
      KeywordFile m;
      if (!m.read(join_dir(hp.dir, f_mode), {"Snapshots", "Solidification"})) { err = "cannot open mode file"; return false; }
      const int ns = m.count("Snapshots"), nsol = m.count("Solidification");
      if (ns + nsol != 1) { err = "the mode file must hold exactly one of Snapshots / Solidification"; return false; }
      bool ok = true;
      hp.dt = 1e-5; hp.out_freq = INT_MAX; hp.rcheck = 1.0;
      if (ns) {
        hp.mode = 0;
        const std::string times = m.str("Snapshots", "Times"), fracs = m.str("Snapshots", "ScanFracs");
        if (!times.empty() && !fracs.empty()) { err = "both Times and ScanFracs given"; return false; }
        std::string item;
        if (!times.empty()) { std::stringstream ss(times); while (std::getline(ss, item, ',')) hp.snaps.push_back(std::stod(item)); }
        if (!fracs.empty()) { std::stringstream ss(fracs); while (std::getline(ss, item, ',')) hp.snaps.push_back(std::stod(item) / 100.0 * hp.end_time); }
        hp.tracking = parse_tracking(m.str("Snapshots", "Tracking"), ok);
        if (!ok) { err = "snapshot tracking modes other than None are not supported"; return false; }
        // other modes are refused once the domain is read: custom points go without tracking
      } else {
        hp.mode = 1;
        hp.tracking = parse_tracking(m.str("Solidification", "Tracking"), ok);
        if (!ok) { err = "unsupported solidification tracking " + m.str("Solidification", "Tracking"); return false; }
        hp.dt = m.num("Solidification", "Timestep", 1e-5);
        hp.out_freq = m.integer("Solidification", "OutputFrequency", INT_MAX);
        hp.rcheck = m.num("Solidification", "CheckRadius", 1.0);
        if (m.flag("Solidification", "Secondary", false)) { err = "secondary solidification is not supported"; return false; }
      }
    }
    // domain (src/Init.cpp:627-707), scan bounds (src/Util.cpp:82-136)
    {
      KeywordFile d;
      const std::string f_dom = top.str("Options", "Domain");
      if (!f_dom.empty()) d.read(join_dir(hp.dir, f_dom), {"X", "Y", "Z", "BoundaryConditions", "Custom"});
      hp.xmin = d.num("X", "Min", -DBL_MAX); hp.xmax = d.num("X", "Max", DBL_MAX); hp.nx = d.integer("X", "Num", INT_MAX); hp.xres = d.num("X", "Res", 50e-6);
      hp.ymin = d.num("Y", "Min", -DBL_MAX); hp.ymax = d.num("Y", "Max", DBL_MAX); hp.ny = d.integer("Y", "Num", INT_MAX); hp.yres = d.num("Y", "Res", 50e-6);
      hp.zmin = d.num("Z", "Min", -DBL_MAX); hp.zmax = d.num("Z", "Max", DBL_MAX); hp.nz = d.integer("Z", "Num", INT_MAX); hp.zres = d.num("Z", "Res", 50e-6);
      hp.bcx0 = d.num("BoundaryConditions", "X_min", DBL_MAX); hp.bcx1 = d.num("BoundaryConditions", "X_max", DBL_MAX);
      hp.bcy0 = d.num("BoundaryConditions", "Y_min", DBL_MAX); hp.bcy1 = d.num("BoundaryConditions", "Y_max", DBL_MAX);
      hp.bcz0 = d.num("BoundaryConditions", "Z_min", DBL_MAX); hp.bc_refl = d.integer("BoundaryConditions", "Reflections", INT_MAX);
      hp.use_bcs = hp.bcx0 != DBL_MAX || hp.bcx1 != DBL_MAX || hp.bcy0 != DBL_MAX || hp.bcy1 != DBL_MAX || hp.bcz0 != DBL_MAX;
      // custom points (src/Init.cpp:686-703), read as Init::FileRead_Points does
      // (src/Init.cpp:816-857): the first line is skipped; then, point by point, the rest of
      // the current line is skipped and three numbers are read (mm), until a read fails
      const std::string f_pts = d.str("Custom", "File");
      hp.custom = !f_pts.empty();
      hp.px.clear(); hp.py.clear(); hp.pz.clear();
      if (hp.custom) {
        std::ifstream in(join_dir(hp.dir, f_pts));
        if (!in) { err = "cannot open the points file " + f_pts; return false; }
        std::string line;
        double x = 0, y = 0, z = 0;
        while (std::getline(in, line) && (in >> x >> y >> z)) {
          hp.px.push_back(x / 1000.0); hp.py.push_back(y / 1000.0); hp.pz.push_back(z / 1000.0);
        }
        if (hp.px.empty()) { err = "no points found in " + f_pts; return false; }
      }

      double sx0 = DBL_MAX, sx1 = -DBL_MAX, sy0 = DBL_MAX, sy1 = -DBL_MAX, sz0 = DBL_MAX, sz1 = -DBL_MAX;
      double px = 0, py = 0, pz = 0, pq = 0;
      bool first = true;
      for (const auto& path : hp.paths) for (const DevSeg& s : path) {
        if (s.q > 0.0) {
          if (first) { sx0 = sx1 = s.x; sy0 = sy1 = s.y; sz0 = sz1 = s.z; }
          else {
            sx0 = std::min(sx0, s.x); sx1 = std::max(sx1, s.x); sy0 = std::min(sy0, s.y); sy1 = std::max(sy1, s.y);
            sz0 = std::min(sz0, s.z); sz1 = std::max(sz1, s.z);
            if (pq == 0.0 && s.mode == 0) {   // the start of a lit line is also scanned
              sx0 = std::min(sx0, px); sx1 = std::max(sx1, px); sy0 = std::min(sy0, py); sy1 = std::max(sy1, py);
              sz0 = std::min(sz0, pz); sz1 = std::max(sz1, pz);
            }
          }
        }
        first = false; px = s.x; py = s.y; pz = s.z; pq = s.q;
      }
      if (hp.xmin == -DBL_MAX) hp.xmin = sx0 - 500e-6;
      if (hp.xmax == DBL_MAX) hp.xmax = sx1 + 500e-6;
      if (hp.ymin == -DBL_MAX) hp.ymin = sy0 - 500e-6;
      if (hp.ymax == DBL_MAX) hp.ymax = sy1 + 500e-6;
      if (hp.zmin == -DBL_MAX) hp.zmin = sz0 - 250e-6;
      if (hp.zmax == DBL_MAX) hp.zmax = sz1;
      if (hp.custom) {
        // no grid (src/Init.cpp:866-869): the points are the list, laid out as pnum x 1 x 1;
        // such a run goes without tracking (src/Run.cpp:61, 391)
        if (hp.px.size() > (size_t)INT_MAX) { err = "too many custom points"; return false; }
        hp.nx = (int)hp.px.size(); hp.ny = hp.nz = 1;
        hp.pnum = (int64_t)hp.px.size();
        hp.tracking = TH_TRACK_NONE;
      } else {
        axis(hp.nx, hp.xmin, hp.xmax, hp.xres, hp.nx == 1);
        axis(hp.ny, hp.ymin, hp.ymax, hp.yres, hp.ny == 1);
        axis(hp.nz, hp.zmin, hp.zmax, hp.zres, hp.ny == 1);
        if (hp.nx < 1 || hp.ny < 1 || hp.nz < 1 || hp.nx > 65535 || hp.ny > 65535 || hp.nz > 65535) {
          err = "grid axis counts must be within 1..65535"; return false;
        }
        hp.pnum = (int64_t)hp.nx * hp.ny * hp.nz;
        if (hp.mode == 0 && hp.tracking != TH_TRACK_NONE) {
          err = "snapshot tracking modes other than None are not supported"; return false;
        }
      }
    }
    // outputs (src/Init.cpp:709-771)
    {
      KeywordFile o;
      const std::string f_out = top.str("Options", "Output");
      if (!f_out.empty()) o.read(join_dir(hp.dir, f_out), {"Grid", "Temperature", "Solidification", "Solidification+"});
      hp.o_x = o.flag("Grid", "x", true); hp.o_y = o.flag("Grid", "y", true); hp.o_z = o.flag("Grid", "z", true);
      hp.o_T = o.flag("Temperature", "T", true);
      // the temperature history (Grid::Output_T_hist, src/Grid.cpp:101-174): without tracking
      // every point is evaluated at the same times and the history is one table; tracked runs'
      // per-point histories are not kept
      hp.o_T_hist = o.flag("Temperature", "T_hist", false);
      if (hp.o_T_hist && hp.tracking != TH_TRACK_NONE) { err = "T_hist output needs Tracking None"; return false; }
      hp.o_tSol = o.flag("Solidification", "tSol", false); hp.o_G = o.flag("Solidification", "G", false);
      hp.o_Gx = o.flag("Solidification", "Gx", false); hp.o_Gy = o.flag("Solidification", "Gy", false);
      hp.o_Gz = o.flag("Solidification", "Gz", false); hp.o_V = o.flag("Solidification", "V", false);
      hp.o_dTdt = o.flag("Solidification", "dTdt", false); hp.o_eqFrac = o.flag("Solidification", "eqFrac", false);
      hp.o_depth = o.flag("Solidification", "depth", false); hp.o_numMelt = o.flag("Solidification", "numMelt", false);
      hp.o_rdf = o.flag("Solidification", "RDF", false);
      if (o.flag("Solidification", "MP_Stats", false)) { err = "MP_Stats output is not supported"; return false; }
      // every solidification output, RDF too, turns the solidification fields on (src/Grid.h:180-241)
      hp.do_sol = hp.mode == 1 && (hp.o_tSol || hp.o_G || hp.o_V || hp.o_Gx || hp.o_Gy || hp.o_Gz || hp.o_dTdt ||
                                   hp.o_eqFrac || hp.o_rdf);
    }
    // settings (src/Init.cpp:772-814) and r_max (src/Util.cpp:145-166)
    {
      KeywordFile s;
      const std::string f_set = top.str("Options", "Settings");
      if (!f_set.empty()) s.read(join_dir(hp.dir, f_set), {"Temperature", "Path", "Compute", "MPI"});
      hp.sol_tol = s.num("Temperature", "Sol_Tol", 1e-3);
      hp.sol_iter = s.integer("Temperature", "Sol_Iter", 10);
      hp.t_hist = s.num("Temperature", "Cutoff_Peak", 1e-9);
      hp.p_hist = s.num("Temperature", "Cutoff_T0TL", 1e-2);
      hp.r_max = s.num("Path", "Buffer", -1.0);
      hp.compress = s.integer("Path", "Compression", 0) != 0;
      hp.t_hist = 1.0 / hp.t_hist;
      if (hp.r_max < 0.0) {
        // as in the reference, the last beam's radius wins
        for (const HostBeam& B : hp.beams) {
          if (hp.t_hist < std::exp(3.0 / 2.0)) hp.r_max = B.ax * std::sqrt(std::log(hp.t_hist) / 3.0);
          else hp.r_max = B.ax * std::pow(hp.t_hist, (1.0 / 3.0)) / std::sqrt(2.0 * std::exp(1.0));
          const double beta = std::pow(3.0 / 3.14159, 1.5) * B.q / (hp.rho * hp.cps);
          const double x = (hp.TL - hp.T0) * hp.p_hist;
          double r2;
          if (beta / (x * B.ax * B.ax * B.ax) < std::exp(3.0 / 2.0)) r2 = B.ax * std::sqrt(std::log(beta / (x * B.ax * B.ax * B.ax)) / 3.0);
          else r2 = std::pow(beta / x, (1.0 / 3.0)) / std::sqrt(2.0 * std::exp(1.0));
          hp.r_max = std::max(hp.r_max, r2);
        }
      }
    }
  } catch (const std::exception& e) {
    err = std::string("malformed value in deck: ") + e.what();
    return false;
  }
  return true;
}

std::vector<DevSeg> th_pack_segments(const HostProblem& hp) {
  std::vector<DevSeg> all;
  for (size_t b = 0; b < hp.paths.size(); ++b)
    for (DevSeg s : hp.paths[b]) {
      // the line-mode step scale of Util::GetRefTime (src/Util.cpp:199), same operations
      s.rt0 = (s.mode == 0) ? 0.58870501125 * hp.beams[b].ax / s.prm : 0.0;
      all.push_back(s);
    }
  return all;
}

void th_make_dev_problem(const HostProblem& hp, const DevSeg* d_segs, DevProblem& dp) {
  dp = DevProblem();
  dp.segs = d_segs;
  dp.nbeams = (int32_t)hp.beams.size();
  int off = 0;
  for (int b = 0; b < dp.nbeams; ++b) {
    const HostBeam& B = hp.beams[b];
    DevBeam& D = dp.beam[b];
    D.ax = B.ax; D.ay = B.ay; D.az = B.az;
    D.ax2 = B.ax * B.ax; D.ay2 = B.ay * B.ay; D.az2 = B.az * B.az;
    D.nond = B.nond;
    D.beta = std::pow(3.0 / kPi, 1.5) * B.q / (hp.rho * hp.cps);   // src/Calc.cpp:96
    D.tlast = hp.paths[b].back().tend;
    D.seg_off = off;
    D.nseg = (int32_t)hp.paths[b].size();
    off += D.nseg;
  }
  dp.T0 = hp.T0; dp.TL = hp.TL; dp.a = hp.a; dp.a12 = 12.0 * hp.a;
  dp.compress = hp.compress ? 1 : 0;
  {  // TL - T0 = s + e exactly (TwoSum); s + e split into three floats
    const double s = hp.TL - hp.T0, bb = s - hp.TL;
    const double e = (hp.TL - (s - bb)) + (-hp.T0 - bb);
    const float f0 = (float)s;
    const double r1 = (s - (double)f0) + e;
    const float f1 = (float)r1;
    const float f2 = (float)(r1 - (double)f1);
    dp.tl_df[0] = f0; dp.tl_df[1] = f1; dp.tl_df[2] = f2;
  }
  dp.cetN0 = hp.cetN0; dp.cetn = hp.cetn; dp.ceta = hp.ceta;
  dp.cx = dp.cy = dp.cz = nullptr;          // set by the context for custom points
  dp.nx = hp.nx; dp.ny = hp.ny; dp.nz = hp.nz;
  udiv_magic((uint32_t)std::max(1, hp.nz), dp.div_nz_m, dp.div_nz_s);
  udiv_magic((uint32_t)std::max(1, hp.ny), dp.div_ny_m, dp.div_ny_s);
  dp.gx = (uint16_t)hp.nx; dp.gy = (uint16_t)hp.ny; dp.gz = (uint16_t)hp.nz;
  dp.pnum = hp.pnum;
  dp.xmin = hp.xmin; dp.xmax = hp.xmax; dp.ymin = hp.ymin; dp.ymax = hp.ymax; dp.zmin = hp.zmin; dp.zmax = hp.zmax;
  dp.xres = hp.xres; dp.yres = hp.yres; dp.zres = hp.zres;
  dp.hx = dp.gx > 1 ? (hp.xmax - hp.xmin) / (dp.gx - 1) : 0.0;
  dp.hy = dp.gy > 1 ? (hp.ymax - hp.ymin) / (dp.gy - 1) : 0.0;
  dp.hz = dp.gz > 1 ? (hp.zmax - hp.zmin) / (dp.gz - 1) : 0.0;
  dp.rx0 = hp.xmin - hp.r_max; dp.rx1 = hp.xmax + hp.r_max;
  dp.ry0 = hp.ymin - hp.r_max; dp.ry1 = hp.ymax + hp.r_max;
  // method-of-images list (src/Calc.cpp:503-582): breadth-first reflections across the
  // given planes, image 0 first; the top plane is always z = zmax and never re-enters 1
  dp.bcx0 = hp.bcx0; dp.bcx1 = hp.bcx1; dp.bcy0 = hp.bcy0; dp.bcy1 = hp.bcy1; dp.bcz0 = hp.bcz0; dp.bcz1 = hp.zmax;
  std::vector<std::vector<int>> all{{0, 0, 0}};
  if (hp.use_bcs) {
    std::vector<std::vector<int>> frontier{{0, 0, 0}};
    const int strength = hp.bc_refl != INT_MAX ? hp.bc_refl : 0;
    auto add = [&](std::vector<int> c, std::vector<std::vector<int>>& fresh, bool top) {
      if (std::find(all.begin(), all.end(), c) != all.end()) return;
      if (top && c[2] == 1) return;
      all.push_back(c); fresh.push_back(c);
    };
    for (int it = 0; !frontier.empty() && it < strength; ++it) {
      std::vector<std::vector<int>> fresh;
      for (const auto& c0 : frontier) {
        std::vector<int> c;
        if (hp.bcx0 != DBL_MAX) { c = c0; c[0] = -1 - c[0]; add(c, fresh, false); }
        if (hp.bcx1 != DBL_MAX) { c = c0; c[0] = 1 - c[0]; add(c, fresh, false); }
        if (hp.bcy0 != DBL_MAX) { c = c0; c[1] = -1 - c[1]; add(c, fresh, false); }
        if (hp.bcy1 != DBL_MAX) { c = c0; c[1] = 1 - c[1]; add(c, fresh, false); }
        if (hp.bcz0 != DBL_MAX) { c = c0; c[2] = -1 - c[2]; add(c, fresh, false); }
        if (hp.zmax != DBL_MAX) { c = c0; c[2] = 1 - c[2]; add(c, fresh, true); }
      }
      frontier.swap(fresh);
    }
  }
  // n_images may exceed TH_MAX_IMAGES; the context rejects such decks before any launch
  dp.n_images = (int32_t)all.size();
  for (int i = 0; i < dp.n_images && i < TH_MAX_IMAGES; ++i) { dp.img[i][0] = all[i][0]; dp.img[i][1] = all[i][1]; dp.img[i][2] = all[i][2]; }
  dp.dt = hp.dt; dp.sol_tol = hp.sol_tol; dp.sol_iter = hp.sol_iter;
  dp.tracking = hp.tracking; dp.rcheck = hp.rcheck; dp.end_time = hp.end_time;
  for (int b = 0; b < dp.nbeams; ++b) {   // src/Melt.cpp:24-31, rounded step by step as there
    DevBeam& D = dp.beam[b];
    const double rc2 = hp.rcheck * hp.rcheck;
    D.tsub = ((rc2 - 1.0) * D.ax2) / (12.0 * dp.a);
    D.r2 = (rc2 * D.ax) * D.ax;
  }
  th_gauss_tables(dp.gl_loc, dp.gl_w);
}
