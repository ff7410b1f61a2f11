// Solution files in the reference's layout (see fv2d_output.cpp).
#pragma once

#include <string>

#include "fv2d_host.h"

namespace fv2d {
int write_mesh_files(const HostMesh& m, const std::string& dir, std::string& err);
int write_history_headers(const std::string& dir, std::string& err);
int save_solution(const HostMesh& m, const fv2d_case& cs, int ndx, const double* q, const double* g, const double* r,
                  const std::string& dir, std::string& err);
int write_restart(const HostMesh& m, int ndx, const double* q, const std::string& dir, std::string& err);
int write_restart_file(const HostMesh& m, const std::string& path, int ndx, const double* q, int digits,
                       std::string& err);
int read_restart(const char* path, int num_cells, int* ndx, double* q, std::string& err);
}  // namespace fv2d
