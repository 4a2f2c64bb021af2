// CSV output in the reference's layout (src/Grid.cpp:72-99, column order from the Grid
// constructor, src/Grid.h:138-254): a header of the enabled field names, then one row
// per output point in point order, every value printed as an ostream would print a double
// with the default precision of 6 significant digits.
#include "th_output.h"

#include <sys/stat.h>
#include <sys/types.h>

#include <cstdio>
#include <string>

std::string th_data_dir(const HostProblem& hp) { return hp.dir + "/Data"; }

bool th_write_csv(const HostProblem& hp, const std::string& tag, const std::vector<std::string>& names,
                  const std::vector<const double*>& cols, const unsigned char* flag, std::string& err) {
  if (names.empty()) return true;
  const std::string dir = th_data_dir(hp);
  mkdir(dir.c_str(), 0777);
  const std::string path = dir + "/" + hp.name + "." + tag + ".csv";
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) { err = "cannot write " + path; return false; }
  std::vector<char> buf(1 << 20);
  std::setvbuf(f, buf.data(), _IOFBF, buf.size());
  for (size_t c = 0; c < names.size(); ++c) std::fprintf(f, c ? ",%s" : "%s", names[c].c_str());
  std::fputc('\n', f);
  const int64_t n = hp.pnum;
  for (int64_t p = 0; p < n; ++p) {
    if (flag && !flag[p]) continue;
    for (size_t c = 0; c < cols.size(); ++c) std::fprintf(f, c ? ",%g" : "%g", cols[c][p]);
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  if (!ok) err = "error writing " + path;
  return ok;
}

// Stork's doubly reduced data (Grid::Output_RRDF_csv, src/Grid.cpp:203-238): the header,
// then per row the cell index, the two step times and the 8 + 8 vertex temperatures.
bool th_write_rrdf_csv(const HostProblem& hp, const std::string& tag, const uint32_t* idx, const double* ts,
                       const double* Ts, int64_t rows, std::string& err) {
  const std::string dir = th_data_dir(hp);
  mkdir(dir.c_str(), 0777);
  const std::string path = dir + "/" + hp.name + "." + tag + ".csv";
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) { err = "cannot write " + path; return false; }
  std::vector<char> buf(1 << 20);
  std::setvbuf(f, buf.data(), _IOFBF, buf.size());
  std::fputs("x,y,z,t_prev,t_cur", f);
  for (int t = 0; t < 2; ++t)
    for (int v = 0; v < 8; ++v) std::fprintf(f, ",T%d%d%d_%s", v >> 2, (v >> 1) & 1, v & 1, t ? "cur" : "prev");
  std::fputc('\n', f);
  for (int64_t r = 0; r < rows; ++r) {
    std::fprintf(f, "%u,%u,%u,%g,%g", idx[3 * r], idx[3 * r + 1], idx[3 * r + 2], ts[2 * r], ts[2 * r + 1]);
    for (int v = 0; v < 16; ++v) std::fprintf(f, ",%g", Ts[16 * r + v]);
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  if (!ok) err = "error writing " + path;
  return ok;
}

// The temperature history without tracking (Grid::Output_T_hist, src/Grid.cpp:101-136): the
// file is <name><tag>.csv (no dot between them, as the reference names it); the header is
// x,y,z and one column per evaluation time, each row a point's coordinates (ostream's default
// 6 significant digits) and its temperatures, times and temperatures as std::to_string prints a
// double (6 decimals).  T holds nt rows of pnum values.
bool th_write_T_hist_csv(const HostProblem& hp, const std::string& tag, const double* t, const double* T, int64_t nt,
                         std::string& err) {
  const std::string dir = th_data_dir(hp);
  mkdir(dir.c_str(), 0777);
  const std::string path = dir + "/" + hp.name + tag + ".csv";
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) { err = "cannot write " + path; return false; }
  std::vector<char> buf(1 << 20);
  std::setvbuf(f, buf.data(), _IOFBF, buf.size());
  std::fputs("x,y,z", f);
  for (int64_t i = 0; i < nt; ++i) std::fprintf(f, ",%f", t[i]);
  std::fputc('\n', f);
  for (int64_t p = 0; p < hp.pnum; ++p) {
    double x, y, z;
    th_point_coord(hp, p, x, y, z);
    std::fprintf(f, "%g,%g,%g", x, y, z);
    for (int64_t i = 0; i < nt; ++i) std::fprintf(f, ",%f", T[i * hp.pnum + p]);
    std::fputc('\n', f);
  }
  const bool ok = std::fclose(f) == 0;
  if (!ok) err = "error writing " + path;
  return ok;
}

// Stork's doubly reduced data as a binary file (Grid::Output_RRDF_bin, src/Grid.cpp:241-273):
// the row count (uint32), the grid's extents (3 x uint32), its origin, x resolution and the
// liquidus (5 x double), then the rows' cell indices (3 x uint32 each), step times (2 x
// double each) and vertex temperatures (16 x double each), in the machine's byte order.
bool th_write_rrdf_bin(const HostProblem& hp, const std::string& tag, const uint32_t* idx, const double* ts,
                       const double* Ts, int64_t rows, std::string& err) {
  if (rows < 0 || rows > (int64_t)UINT32_MAX) { err = "too many rows for the binary file's uint32 count"; return false; }
  const std::string dir = th_data_dir(hp);
  mkdir(dir.c_str(), 0777);
  const std::string path = dir + "/" + hp.name + "." + tag + ".bin";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { err = "cannot write " + path; return false; }
  const uint32_t head[4] = {(uint32_t)rows, (uint32_t)hp.nx, (uint32_t)hp.ny, (uint32_t)hp.nz};
  const double geo[5] = {hp.xmin, hp.ymin, hp.zmin, hp.xres, hp.TL};
  const size_t n = (size_t)rows;
  bool ok = std::fwrite(head, sizeof(uint32_t), 4, f) == 4 && std::fwrite(geo, sizeof(double), 5, f) == 5;
  ok = ok && (n == 0 || (std::fwrite(idx, sizeof(uint32_t), 3 * n, f) == 3 * n &&
                         std::fwrite(ts, sizeof(double), 2 * n, f) == 2 * n &&
                         std::fwrite(Ts, sizeof(double), 16 * n, f) == 16 * n));
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) err = "error writing " + path;
  return ok;
}

// The reference's reduced data (Grid::Output_RDF, src/Grid.cpp:176-201): the header, then per
// row the point's coordinates, melting time, solidification time and cooling rate.
bool th_write_rdf_csv(const HostProblem& hp, const std::string& tag, const int64_t* pts, const double* tm,
                      const double* tl, const double* cr, int64_t rows, std::string& err) {
  const std::string dir = th_data_dir(hp);
  mkdir(dir.c_str(), 0777);
  const std::string path = dir + "/" + hp.name + "." + tag + ".csv";
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) { err = "cannot write " + path; return false; }
  std::vector<char> buf(1 << 20);
  std::setvbuf(f, buf.data(), _IOFBF, buf.size());
  std::fputs("x,y,z,tm,tl,cr\n", f);
  for (int64_t r = 0; r < rows; ++r) {
    double x, y, z;
    th_point_coord(hp, pts[r], x, y, z);
    std::fprintf(f, "%g,%g,%g,%g,%g,%g\n", x, y, z, tm[r], tl[r], cr[r]);
  }
  const bool ok = std::fclose(f) == 0;
  if (!ok) err = "error writing " + path;
  return ok;
}

void th_point_coord(const HostProblem& hp, int64_t p, double& x, double& y, double& z) {
  if (hp.custom) { x = hp.px[p]; y = hp.py[p]; z = hp.pz[p]; return; }
  const int gx = (uint16_t)hp.nx, gy = (uint16_t)hp.ny, gz = (uint16_t)hp.nz;
  const int64_t nyz = (int64_t)hp.ny * hp.nz;
  const int i = (int)(p / nyz), j = (int)((p / hp.nz) % hp.ny), k = (int)(p % hp.nz);
  x = (gx - 1) ? hp.xmin + (double(i) * ((hp.xmax - hp.xmin) / (gx - 1))) : hp.xmax;
  y = (gy - 1) ? hp.ymin + (double(j) * ((hp.ymax - hp.ymin) / (gy - 1))) : hp.ymax;
  z = (gz - 1) ? hp.zmin + (double(k) * ((hp.zmax - hp.zmin) / (gz - 1))) : hp.zmax;
}

void th_grid_coords(const HostProblem& hp, std::vector<double>& x, std::vector<double>& y, std::vector<double>& z) {
  if (hp.custom) { x = hp.px; y = hp.py; z = hp.pz; return; }
  const int gx = (uint16_t)hp.nx, gy = (uint16_t)hp.ny, gz = (uint16_t)hp.nz;
  const double hx = gx > 1 ? (hp.xmax - hp.xmin) / (gx - 1) : 0.0;
  const double hy = gy > 1 ? (hp.ymax - hp.ymin) / (gy - 1) : 0.0;
  const double hz = gz > 1 ? (hp.zmax - hp.zmin) / (gz - 1) : 0.0;
  x.resize(hp.pnum); y.resize(hp.pnum); z.resize(hp.pnum);
  int64_t p = 0;
  for (int i = 0; i < hp.nx; ++i) {
    const double xv = (gx - 1) ? hp.xmin + (double(i) * hx) : hp.xmax;
    for (int j = 0; j < hp.ny; ++j) {
      const double yv = (gy - 1) ? hp.ymin + (double(j) * hy) : hp.ymax;
      for (int k = 0; k < hp.nz; ++k, ++p) {
        x[p] = xv; y[p] = yv;
        z[p] = (gz - 1) ? hp.zmin + (double(k) * hz) : hp.zmax;
      }
    }
  }
}

std::string th_zero_pad(int v, int width) {
  char b[32];
  std::snprintf(b, sizeof(b), "%0*d", width, v);
  return b;
}
