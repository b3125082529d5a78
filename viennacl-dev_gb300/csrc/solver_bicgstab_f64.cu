// bicgstab_solve<double>: one instantiation of the solvers in solvers.cuh.
#include "solvers.cuh"

namespace vclgb {
template void bicgstab_solve<double>(Backend &, Matrix &, const double *, double *, vclgbSolverTag *, const Precond *);
}  // namespace vclgb
