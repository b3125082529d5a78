// Stands in for ViennaCL's viennacl/linalg/cg.hpp: includes the original,
// then declares linalg::solve(compressed_matrix<T>, vector<T>, cg_tag[, precond])
// for T = float, double with no preconditioner, jacobi_precond and ilu0_precond,
// solved in the engine (see vclgb_solvers.hpp).
#ifndef VCLGB_SHADOW_CG_HPP
#define VCLGB_SHADOW_CG_HPP

#include_next <viennacl/linalg/cg.hpp>

#include "vclgb_solvers.hpp"

namespace vclgb_viennacl {

template <typename T>
inline viennacl::vector<T> cg(viennacl::compressed_matrix<T> const &A, viennacl::vector<T> const &b,
                              viennacl::linalg::cg_tag const &tag, int pc) {
  vclgbSolverTag t;
  fill_tag(t, 0, tag.tolerance(), tag.abs_tolerance(), tag.max_iterations());
  viennacl::vector<T> x = solve<T>(0, A, b, t, pc);
  tag.iters(t.iters);
  tag.error(t.error);
  return x;
}

}  // namespace vclgb_viennacl

VCLGB_SHADOW_SOLVE(viennacl::linalg::cg_tag, cg, double)
VCLGB_SHADOW_SOLVE(viennacl::linalg::cg_tag, cg, float)

#endif
