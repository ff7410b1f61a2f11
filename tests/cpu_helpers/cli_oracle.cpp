// Test harness: the fv2d_gpu command-line sequence (csrc/fv2d_cli.cpp) with the ORACLE PORT as the
// stepper and the library's own host output writers (csrc/fv2d_output.cpp).  Checks the writers on
// the CPU against the reference program's golden output files; the product never links the oracle.
#include <cstdio>
#include <filesystem>
#include <iostream>
#include <string>
#include <vector>
#include "fv2d_gpu.h"
#include "fv2d_host.h"
#include "fv2d_output.h"
#include "fv2d_oracle.h"
int main(int argc, char** argv) {
    const char* input = argc > 1 ? argv[1] : "input.in";
    std::filesystem::create_directory("sol");
    std::filesystem::create_directory("mesh");
    fv2d_case cs; std::string err;
    if (fv2d::parse_inputs(input, &cs, err)) { std::cerr << err << "\n"; return 1; }
    std::vector<double> x, y; std::vector<int> a, b, c, d; int nc = 0;
    if (fv2d::parse_grid(cs.grid_file, x, y, a, b, c, d, nc, err)) { std::cerr << err << "\n"; return 1; }
    fv2d_mesh_desc desc{(int)x.size(), (int)a.size(), nc, x.data(), y.data(), a.data(), b.data(), c.data(), d.data()};
    fv2d::HostMesh m;
    if (fv2d::build_mesh(&desc, &cs, m, err)) { std::cerr << err << "\n"; return 1; }
    void* o = fvo_open(input);
    fv2d::write_mesh_files(m, "mesh", err);
    int ndx = 1;
    const int N = m.nc;
    std::vector<double> q(4 * N), g(8 * N), r(4 * N);
    if (cs.restart == 1) {
        int at = 0;
        if (fv2d::read_restart("sol/restart_sol.dat", N, &at, q.data(), err)) { std::cerr << err << "\n"; return 1; }
        fvo_set_state(o, q.data());
        ndx = at + 1;
    } else fv2d::write_history_headers("sol", err);
    for (; ndx <= cs.nmax; ndx++) {
        fvo_iterate(o, 1);
        fvo_get(o, FVO_QBAR, q.data()); fvo_get(o, FVO_QBAR_GRAD, g.data()); fvo_get(o, FVO_RES, r.data());
        if (fv2d::save_solution(m, cs, ndx, q.data(), g.data(), r.data(), "sol", err)) { std::cerr << err << "\n"; return 1; }
    }
    fvo_get(o, FVO_QBAR, q.data());
    fv2d::write_restart(m, cs.nmax, q.data(), "sol", err);
    fvo_close(o);
    return 0;
}
