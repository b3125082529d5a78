// vclgb_viennacl.hpp -- glue between ViennaCL's CUDA types and the engine's C ABI.
//
// The headers under viennacl/ beside this file stand in for ViennaCL's own
// headers of the same names: each includes the original (#include_next) and
// then declares non-template overloads of the backend functions and solver
// entry points for the matrix and vector types the engine serves.  An exact
// non-template overload is preferred to ViennaCL's function templates, so
// viennacl::linalg::prod, inner_prod, norm_2, the vector updates and
// linalg::solve with cg_tag / bicgstab_tag / gmres_tag run in the engine
// (libvclgb.so) while every other ViennaCL function keeps its own code.
//
// Use: compile with  -DVIENNACL_WITH_CUDA  -I<this directory>  -I<repo>/include
// -I<ViennaCL source tree>  (this directory first) and link libvclgb.so.
//
// The engine keeps a handle per matrix (validated and analysed once), keyed by
// the matrix's device buffers and sizes; a matrix whose buffers are rewritten
// with a different pattern must call vclgb_viennacl::forget(matrix) first.
// Failures raise std::runtime_error with the engine's message, as ViennaCL
// raises its own exceptions.
#ifndef VCLGB_VIENNACL_HPP
#define VCLGB_VIENNACL_HPP

#include <cstdint>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>

#include "vclgb.h"

namespace vclgb_viennacl {

struct Context {
  vclgbBackend be = nullptr;
  // (format, ptr0, ptr1, ptr2, rows, cols, nnz) -> matrix handle
  typedef std::tuple<int, const void *, const void *, const void *, uint64_t, uint64_t, uint64_t>
      Key;
  std::map<Key, vclgbMatrix> mats;
  std::map<std::pair<vclgbMatrix, int>, vclgbPrecond> preconds;
  std::mutex mu;
  ~Context() {
    // handles are released at process exit by the driver; nothing to free here
  }
};

inline Context &ctx() {
  static Context c;
  if (!c.be) {
    // a blocking stream: ordered with ViennaCL's legacy-default-stream kernels
    if (vclgbBackendCreate(&c.be, nullptr) != VCLGB_SUCCESS)
      throw std::runtime_error("vclgb: backend creation failed");
  }
  return c;
}

inline void check(vclgbStatus s, const char *what) {
  if (s == VCLGB_SUCCESS || s == VCLGB_NOT_CONVERGED || s == VCLGB_BREAKDOWN) return;
  throw std::runtime_error(std::string("vclgb: ") + what + ": " +
                           vclgbBackendLastError(ctx().be));
}

template <typename T>
inline vclgbPrecision prec() {
  return sizeof(T) == 8 ? VCLGB_FLOAT64 : VCLGB_FLOAT32;
}

// one handle per set of device buffers
template <typename F>
inline vclgbMatrix cached(const Context::Key &k, F &&create) {
  Context &c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  auto it = c.mats.find(k);
  if (it != c.mats.end()) return it->second;
  vclgbMatrix m = create(c.be);
  c.mats[k] = m;
  return m;
}

// the preconditioner object of kind `kind` (0 Jacobi, 1 ILU0) built from m
template <typename F>
inline vclgbPrecond cached_precond(vclgbMatrix m, int kind, F &&create) {
  Context &c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  auto it = c.preconds.find({m, kind});
  if (it != c.preconds.end()) return it->second;
  vclgbPrecond p = create(c.be);
  c.preconds[{m, kind}] = p;
  return p;
}

inline void fill_tag(vclgbSolverTag &t, int kind, double tol, double abs_tol, unsigned max_iters) {
  vclgbSolverTagInit(&t, kind);
  t.tol = tol;
  t.abs_tol = abs_tol;
  t.max_iters = max_iters;
}

}  // namespace vclgb_viennacl

#endif
