#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "th_problem.h"

std::string th_data_dir(const HostProblem& hp);
// Writes <deck dir>/Data/<name>.<tag>.csv; rows only where flag[p] (all rows if flag is null).
bool th_write_csv(const HostProblem& hp, const std::string& tag, const std::vector<std::string>& names,
                  const std::vector<const double*>& cols, const unsigned char* flag, std::string& err);
// Writes <deck dir>/Data/<name>.<tag>.csv with Stork's rows (3 indices, 2 times, 16
// temperatures each).
bool th_write_rrdf_csv(const HostProblem& hp, const std::string& tag, const uint32_t* idx, const double* ts,
                       const double* Ts, int64_t rows, std::string& err);
// Writes <deck dir>/Data/<name><tag>.csv: the temperature history of a run without tracking
// (nt times; T time by time, pnum values each).
bool th_write_T_hist_csv(const HostProblem& hp, const std::string& tag, const double* t, const double* T, int64_t nt,
                         std::string& err);
// Writes <deck dir>/Data/<name>.<tag>.bin: the same rows in the reference's binary layout.
bool th_write_rrdf_bin(const HostProblem& hp, const std::string& tag, const uint32_t* idx, const double* ts,
                       const double* Ts, int64_t rows, std::string& err);
// Writes <deck dir>/Data/<name>.<tag>.csv with the reduced data's rows (point, melting time,
// solidification time, cooling rate).
bool th_write_rdf_csv(const HostProblem& hp, const std::string& tag, const int64_t* pts, const double* tm,
                      const double* tl, const double* cr, int64_t rows, std::string& err);
// One point's coordinates, as th_grid_coords gives them.
void th_point_coord(const HostProblem& hp, int64_t p, double& x, double& y, double& z);
// Point coordinates exactly as the reference's Grid getters compute them.
void th_grid_coords(const HostProblem& hp, std::vector<double>& x, std::vector<double>& y, std::vector<double>& z);
std::string th_zero_pad(int v, int width);
