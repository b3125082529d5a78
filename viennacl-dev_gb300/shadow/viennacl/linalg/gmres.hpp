// Stands in for ViennaCL's viennacl/linalg/gmres.hpp: includes the original,
// then declares linalg::solve(compressed_matrix<T>, vector<T>, gmres_tag[, precond])
// for T = float, double with no preconditioner, jacobi_precond and ilu0_precond,
// solved in the engine (see vclgb_solvers.hpp).
#ifndef VCLGB_SHADOW_GMRES_HPP
#define VCLGB_SHADOW_GMRES_HPP

#include_next <viennacl/linalg/gmres.hpp>

#include "vclgb_solvers.hpp"

namespace vclgb_viennacl {

template <typename T>
inline viennacl::vector<T> gmres(viennacl::compressed_matrix<T> const &A,
                                 viennacl::vector<T> const &b,
                                 viennacl::linalg::gmres_tag const &tag, int pc) {
  vclgbSolverTag t;
  fill_tag(t, 2, tag.tolerance(), tag.abs_tolerance(), tag.max_iterations());
  t.krylov_dim = tag.krylov_dim();
  viennacl::vector<T> x = solve<T>(2, A, b, t, pc);
  tag.iters(t.iters);
  tag.error(t.error);
  return x;
}

}  // namespace vclgb_viennacl

VCLGB_SHADOW_SOLVE(viennacl::linalg::gmres_tag, gmres, double)
VCLGB_SHADOW_SOLVE(viennacl::linalg::gmres_tag, gmres, float)

#endif
