// Host-side mesh model of the GB300 fv2d library: input.in parsing, grid parsing, connectivity,
// geometry (the reference's formulas, evaluated in the same operation order so FP64 results are
// bit-identical when compiled with -ffp-contract=off) and the Hilbert renumbering that gives the
// device its deterministic per-cell gathers.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "fv2d_gpu.h"

namespace fv2d {

struct HostMesh {
    int np = 0, nf = 0, nc = 0;
    int numBC1 = 0, numBC2 = 0, numWALL = -1, num_of_BC = 0, max_sides = 0;
    int bc1 = 0, bc2 = 0;                    // the BC codes the mesh was tagged with
    std::vector<double> x, y;
    // connectivity, reference numbering (0-based; fc2 < 0 is a BC code)
    std::vector<int> fp1, fp2, fc1, fc2;
    std::vector<int> cf_off, cf;            // cell -> faces, ascending face id
    std::vector<int> bc_faces, face2bc;
    // geometry, reference numbering
    std::vector<double> area, nx, ny, fcx, fcy;
    std::vector<double> vol, ccx, ccy, delta, Ixx, Iyy, Ixy;
    std::vector<double> bccx, bccy;
    std::vector<double> c1dx, c1dy, c2dx, c2dy, dxj, dyj;
    std::vector<double> dist, lx, ly, mx, my;
    // renumbering (device order)
    std::vector<int> cell_new2old, cell_old2new, face_new2old, face_old2new;
    // the batch engine's upload image of this mesh (per state precision, built on first admission,
    // freed with the mesh)
    mutable std::shared_ptr<void> batch_image[2];
};

// Device-order arrays derived from a HostMesh (what gets uploaded).
struct DeviceLayout {
    int nc = 0, nf = 0, ninc = 0;
    std::vector<int> inc_off;               // [nc+1]
    std::vector<int> inc;                   // [ninc] (new face id << 1) | side, ascending original face id
    std::vector<int> nbr;                   // [ninc] neighbour (new id) or BC code
    std::vector<double> igeo;               // [4 ninc] per incidence: dxj, dyj, and the face-centre offset
                                            //   from this cell (c1dx, c1dy or c2dx, c2dy), CSR order
    std::vector<int> fc1, fc2;              // [nf]   new cell ids / BC code
    std::vector<int> qcell;                 // [nf]   NO_SLIP gradient ghost cell (new id of cell `orig face id`), else -1
    std::vector<double> vol, Ixx, Iyy, Ixy; // [nc]
    // face geometry [nf]: nx ny area c1dx c1dy c2dx c2dy dxj dyj mx my lx ly dist
    std::vector<double> fgeo[14];
};

int parse_inputs(const char* path, fv2d_case* cs, std::string& err);
int parse_grid(const char* path, std::vector<double>& x, std::vector<double>& y,
               std::vector<int>& fp1, std::vector<int>& fp2, std::vector<int>& fc1,
               std::vector<int>& fc2, int& nc, std::string& err);
int write_grid(const char* path, const fv2d_mesh_desc* d, std::string& err);
int build_mesh(const fv2d_mesh_desc* d, const fv2d_case* cs, HostMesh& m, std::string& err);
void build_layout(const HostMesh& m, DeviceLayout& L);
int mesh_field(const HostMesh& m, int field, double* out);

}  // namespace fv2d
