// Precision-agnostic interface between the C ABI (fv2d_api.cu) and the solver engines
// (fv2d_fp64.cu, fv2d_fp32.cu).
#pragma once

#include <string>

#include "fv2d_gpu.h"
#include "fv2d_host.h"

namespace fv2d {

// K_TSTAGE: the FP32 engine's fused stage kernel (gradient, flux and update of a tile in one launch)
enum KernelId { K_GRADIENT = 0, K_FACE, K_UPDATE, K_SPECTRAL, K_STATE_IN, K_STATE_OUT, K_NORM, K_TSTAGE, K_COUNT };
extern const char* const kKernelNames[K_COUNT];

class Solver {
public:
    virtual ~Solver() {}
    virtual int init(const fv2d_case& cs) = 0;       // mesh_ must be set before
    virtual int stage() = 0;
    virtual int step(int iterations) = 0;
    virtual int set_state(const double* q) = 0;
    virtual int load_state(const double* q) = 0;
    virtual int get_field(int field, double* out) = 0;
    virtual int residual_norm(double out[4]) = 0;
    virtual int synchronize() = 0;
    virtual int set_store_residual(int every) = 0;
    virtual int set_graphs(int enable) = 0;
    virtual int set_timing(int enable) = 0;
    virtual int kernel_times(double* ms, int* launches) = 0;
    virtual void* stream() = 0;
    virtual long long device_bytes() const = 0;
    int current_stage() const { return stage_; }

    HostMesh mesh_;
    std::string err_;
protected:
    int stage_ = 0;
};

Solver* make_solver_fp64();
Solver* make_solver_fp32();

}  // namespace fv2d
