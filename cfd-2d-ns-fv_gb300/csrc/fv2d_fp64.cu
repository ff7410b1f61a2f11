// FP64 engine.  Built with -fmad=false: every a*b+c rounds twice, as in the reference's CPU
// build, so the plain FP64 path is bit-identical to it.
#include "fv2d_batch_impl.cuh"
#include "fv2d_solver_impl.cuh"

namespace fv2d {
Solver* make_solver_fp64() { return new SolverImpl<double>(); }
Batch* make_batch_fp64() { return new BatchImpl<double>(); }
}
