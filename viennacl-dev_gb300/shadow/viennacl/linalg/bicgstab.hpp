// Stands in for ViennaCL's viennacl/linalg/bicgstab.hpp: includes the original,
// then declares linalg::solve(compressed_matrix<T>, vector<T>, bicgstab_tag[, precond])
// for T = float, double with no preconditioner, jacobi_precond and ilu0_precond,
// solved in the engine (see vclgb_solvers.hpp).
#ifndef VCLGB_SHADOW_BICGSTAB_HPP
#define VCLGB_SHADOW_BICGSTAB_HPP

#include_next <viennacl/linalg/bicgstab.hpp>

#include "vclgb_solvers.hpp"

namespace vclgb_viennacl {

template <typename T>
inline viennacl::vector<T> bicgstab(viennacl::compressed_matrix<T> const &A,
                                    viennacl::vector<T> const &b,
                                    viennacl::linalg::bicgstab_tag const &tag, int pc) {
  vclgbSolverTag t;
  fill_tag(t, 1, tag.tolerance(), tag.abs_tolerance(), tag.max_iterations());
  t.max_iters_before_restart = tag.max_iterations_before_restart();
  viennacl::vector<T> x = solve<T>(1, A, b, t, pc);
  tag.iters(t.iters);
  tag.error(t.error);
  return x;
}

}  // namespace vclgb_viennacl

VCLGB_SHADOW_SOLVE(viennacl::linalg::bicgstab_tag, bicgstab, double)
VCLGB_SHADOW_SOLVE(viennacl::linalg::bicgstab_tag, bicgstab, float)

#endif
