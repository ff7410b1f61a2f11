// FP32 engine: state, gradients and fluxes in FP32; the LSQ moments are kept in FP64 and the
// residual norms are accumulated in FP64.  Built with -fmad=false so the single-solve and batched
// kernels, which share the per-element code, give bit-identical results, and with approximate
// division and square root (a few ulp, far inside the path's accuracy target).
#include "fv2d_batch_impl.cuh"
#include "fv2d_solver_impl.cuh"

namespace fv2d {
Solver* make_solver_fp32() { return new SolverImpl<float>(); }
Batch* make_batch_fp32() { return new BatchImpl<float>(); }
}
