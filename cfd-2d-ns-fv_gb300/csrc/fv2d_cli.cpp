// fv2d_gpu: the fv2d command line with the solver step on the GPU.
//
//   fv2d_gpu [--fp32] [input.in]
//
// Same sequence and files as the reference program (src/base/main.cpp:33-140): read input.in
// (default ./input.in) and the grid it names, write mesh/cell_data.dat and mesh/face_data.dat,
// start the history files (or read sol/restart_sol.dat when restart = 1), run iterations up to
// nmax with the monitor / Tecplot output cadence of save(), and write sol/restart_sol.dat.  The
// state stays on the GPU between output events; each event copies back what save() reads.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <iostream>
#include <vector>

#include "fv2d_gpu.h"

namespace {
int die(const char* what, fv2d_handle* h) {
    std::cerr << "ERROR: " << what << ": " << fv2d_last_error(h) << std::endl;
    return 1;
}
bool event(const fv2d_case& cs, int k) {
    return (cs.monitor_step > 0 && k % cs.monitor_step == 0) || (cs.output_step > 0 && k % cs.output_step == 0);
}
}  // namespace

int main(int argc, char** argv) {
    int precision = FV2D_FP64;
    const char* input = "input.in";
    for (int i = 1; i < argc; i++) {
        if (std::strcmp(argv[i], "--fp32") == 0) precision = FV2D_FP32;
        else input = argv[i];
    }
    try {
        std::filesystem::create_directory("sol");
        std::filesystem::create_directory("mesh");
    } catch (const std::exception&) {
    }
    fv2d_case cs;
    if (fv2d_read_inputs(input, &cs)) return die("cannot read the input file", nullptr);
    std::cout << "Reading " << cs.grid_file << std::endl;
    fv2d_handle* h = nullptr;
    if (fv2d_create_from_files(input, precision, &h)) return die("cannot set up the solve", nullptr);
    int sz[8];
    fv2d_sizes(h, sz);
    std::cout << sz[0] << " Points \n" << sz[1] << " Faces \n" << sz[2] << " Cells \n";
    if (fv2d_write_mesh_files(h)) std::cerr << "ERROR: Cannot Save File \n";
    int ndx = 1;
    if (cs.restart == 1) {
        std::vector<double> q(4 * (size_t)sz[2]);
        int at = 0;
        if (fv2d_read_restart("sol/restart_sol.dat", sz[2], &at, q.data())) return die("restart", h);
        if (fv2d_set_state(h, q.data())) return die("restart state", h);
        ndx = at + 1;
    } else if (fv2d_write_history_headers(h)) {
        return die("history files", h);
    }
    while (ndx <= cs.nmax) {
        int e = ndx;
        while (e < cs.nmax && !event(cs, e)) e++;
        if (fv2d_step(h, e - ndx + 1)) return die("step", h);
        if (event(cs, e)) {
            const int rc = fv2d_save(h, e);
            if (rc == FV2D_ERR_STATE) std::cerr << "WARNING: " << fv2d_last_error(h) << std::endl;
            else if (rc) return die("save", h);
        }
        ndx = e + 1;
    }
    if (fv2d_synchronize(h) == FV2D_ERR_STATE) std::cerr << "WARNING: " << fv2d_last_error(h) << std::endl;
    const int rc = fv2d_post(h, cs.nmax);
    if (rc && rc != FV2D_ERR_STATE) return die("restart file", h);
    fv2d_destroy(h);
    return 0;
}
