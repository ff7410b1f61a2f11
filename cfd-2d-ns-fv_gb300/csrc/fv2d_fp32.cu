// FP32 engine: state, gradients and fluxes in FP32 (FMA contraction allowed); the LSQ moments
// are kept in FP64 and the residual norms are accumulated in FP64.
#include "fv2d_solver_impl.cuh"

namespace fv2d {
Solver* make_solver_fp32() { return new SolverImpl<float>(); }
}
