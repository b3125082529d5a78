// vclgb_solvers.hpp -- linalg::solve(compressed_matrix<T>, vector<T>, tag[, precond])
// overloads for cg_tag, bicgstab_tag and gmres_tag with no preconditioner, the
// Jacobi preconditioner and ILU0: the whole solve (SpMV, reductions, scalar
// recurrences, stopping test) runs in the engine (vclgbSolveCG /
// vclgbSolveBiCGStab / vclgbSolveGMRES) with the reference's stopping tests;
// the tag's iters() and error() are set as the reference's solvers set them.
// Included by the shadow cg.hpp, bicgstab.hpp and gmres.hpp after the
// originals (viennacl/linalg/cg.hpp:338-375, bicgstab.hpp:495-533,
// gmres.hpp:635-673 are the templates these overloads win over).
#ifndef VCLGB_SHADOW_SOLVERS_HPP
#define VCLGB_SHADOW_SOLVERS_HPP

#include <viennacl/compressed_matrix.hpp>
#include <viennacl/linalg/cuda/sparse_matrix_operations.hpp>
#include <viennacl/linalg/detail/ilu/ilu0.hpp>
#include <viennacl/linalg/jacobi_precond.hpp>
#include <viennacl/vector.hpp>

#include "vclgb_viennacl.hpp"

namespace vclgb_viennacl {

enum { kNoPrecond = -1, kJacobi = 0, kIlu0 = 1 };

// kind 0 CG, 1 BiCGStab, 2 GMRES; pc: kNoPrecond, kJacobi, kIlu0
template <typename T>
inline viennacl::vector<T> solve(int kind, viennacl::compressed_matrix<T> const &A,
                                 viennacl::vector<T> const &b, vclgbSolverTag &t, int pc) {
  Context &c = ctx();
  vclgbMatrix M = handle_of(A);
  vclgbPrecond P = nullptr;
  if (pc == kJacobi)
    P = cached_precond(M, kJacobi, [&](vclgbBackend be) {
      vclgbPrecond p = nullptr;
      check(vclgbJacobiCreate(be, M, &p), "jacobi_precond");
      return p;
    });
  else if (pc == kIlu0)
    P = cached_precond(M, kIlu0, [&](vclgbBackend be) {
      vclgbPrecond p = nullptr;
      check(vclgbIlu0Create(be, M, 1, &p), "ilu0_precond");
      return p;
    });
  viennacl::vector<T> x(b.size(), viennacl::traits::context(b));
  const void *pb = viennacl::cuda_arg(b);
  void *px = viennacl::cuda_arg(x);
  // ViennaCL filled b on the legacy default stream; the backend's blocking
  // stream is ordered after it
  if (kind == 0) check(vclgbSolveCG(c.be, M, pb, px, &t, P), "cg");
  else if (kind == 1) check(vclgbSolveBiCGStab(c.be, M, pb, px, &t, P), "bicgstab");
  else check(vclgbSolveGMRES(c.be, M, pb, px, &t, P), "gmres");
  return x;
}

}  // namespace vclgb_viennacl

#define VCLGB_SHADOW_SOLVE(TAG, FN, T)                                                        \
  namespace viennacl {                                                                        \
  namespace linalg {                                                                          \
  inline viennacl::vector<T> solve(viennacl::compressed_matrix<T> const &A,                   \
                                   viennacl::vector<T> const &b, TAG const &tag,              \
                                   viennacl::linalg::no_precond const &) {                    \
    return vclgb_viennacl::FN<T>(A, b, tag, vclgb_viennacl::kNoPrecond);                      \
  }                                                                                           \
  inline viennacl::vector<T> solve(                                                           \
      viennacl::compressed_matrix<T> const &A, viennacl::vector<T> const &b, TAG const &tag,  \
      viennacl::linalg::jacobi_precond<viennacl::compressed_matrix<T> > const &) {            \
    return vclgb_viennacl::FN<T>(A, b, tag, vclgb_viennacl::kJacobi);                         \
  }                                                                                           \
  inline viennacl::vector<T> solve(                                                           \
      viennacl::compressed_matrix<T> const &A, viennacl::vector<T> const &b, TAG const &tag,  \
      viennacl::linalg::ilu0_precond<viennacl::compressed_matrix<T> > const &) {              \
    return vclgb_viennacl::FN<T>(A, b, tag, vclgb_viennacl::kIlu0);                           \
  }                                                                                           \
  inline viennacl::vector<T> solve(viennacl::compressed_matrix<T> const &A,                   \
                                   viennacl::vector<T> const &b, TAG const &tag) {            \
    return vclgb_viennacl::FN<T>(A, b, tag, vclgb_viennacl::kNoPrecond);                      \
  }                                                                                           \
  }                                                                                           \
  }

#endif
