// cg_solve<float>: one instantiation of the solvers in solvers.cuh.
#include "solvers.cuh"

namespace vclgb {
template void cg_solve<float>(Backend &, Matrix &, const float *, float *, vclgbSolverTag *, const Precond *);
}  // namespace vclgb
