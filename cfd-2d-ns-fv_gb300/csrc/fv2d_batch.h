// Precision-agnostic interface of the batched engine: many independent solves resident in one
// device arena, advanced together by persistent tile kernels (one launch per kernel per RK stage,
// one CUDA graph per iteration).  Solves can join and leave between iterations.
#pragma once

#include <string>
#include <vector>

#include "fv2d_gpu.h"
#include "fv2d_host.h"

namespace fv2d {

struct BatchTuning {
    int block = 256;              // threads per block of the persistent kernels
    int tile_mult[3] = {1, 2, 4}; // tile = block * mult elements, per size bucket (small, medium, large)
    int bucket_edges[2] = {16384, 131072};   // cells
    int full_grid = 0;            // 0: persistent grid (SMs x resident blocks); 1: one block per tile
};

class Batch {
public:
    virtual ~Batch() {}
    virtual int init(long long max_cells, long long max_faces, int max_solves) = 0;
    virtual int add(const fv2d_mesh_desc* d, const fv2d_case* cs, int* sid) = 0;
    virtual int add_mesh(const HostMesh& hm, const fv2d_case* cs, int* sid) = 0;
    virtual int remove(int sid) = 0;
    virtual int step(int iterations) = 0;
    virtual int norms(int* sids, double* out, int* iters, int max, int* n) = 0;
    virtual int get_state(int sid, double* q) = 0;
    virtual int synchronize() = 0;
    virtual int set_tuning(const BatchTuning& t) = 0;
    virtual BatchTuning tuning() const = 0;
    virtual int usage(long long* out8) = 0;
    virtual int set_timing(int enable) = 0;
    virtual int kernel_times(double* ms, int* launches) = 0;
    virtual void* stream() = 0;
    std::string err_;
};

Batch* make_batch_fp64();
Batch* make_batch_fp32();

// Device bytes a solve occupies: per cell, per face, per incidence (both precisions).
void batch_footprint(int precision, long long cells, long long faces, long long incs, long long* bytes);
// The FP32 engine's allowance for a solve of `cells` cells and `faces` faces (its tile layout).
void tiled_footprint(long long cells, long long faces, long long* bytes);

}  // namespace fv2d
