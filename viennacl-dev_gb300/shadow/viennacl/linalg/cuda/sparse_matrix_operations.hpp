// Stands in for ViennaCL's viennacl/linalg/cuda/sparse_matrix_operations.hpp:
// includes the original, then routes y = alpha*A*x + beta*y
// (viennacl::linalg::cuda::prod_impl, original :262-396, :1321-1349, :1796-1838,
// :2247-2289, :2357-2403) for compressed_matrix, coordinate_matrix, ell_matrix,
// sliced_ell_matrix and hyb_matrix of float and double, and the CSR triangular
// solves inplace_solve(A | trans(A), vec, tag) (original :778-1008), to the
// engine's C ABI.  The reference's dispatcher
// (viennacl/linalg/sparse_matrix_operations.hpp:101-120, 258-316) calls these
// overloads, which are more specialised than its templates.
#ifndef VCLGB_SHADOW_CUDA_SPARSE_MATRIX_OPERATIONS_HPP
#define VCLGB_SHADOW_CUDA_SPARSE_MATRIX_OPERATIONS_HPP

#include_next <viennacl/linalg/cuda/sparse_matrix_operations.hpp>

#include <cuda_runtime.h>

#include "vclgb_viennacl.hpp"

namespace vclgb_viennacl {

template <typename T>
inline const void *dev(viennacl::backend::mem_handle const &h) {
  return viennacl::cuda_arg<T>(h);
}

template <typename T, unsigned int A>
inline vclgbMatrix handle_of(viennacl::compressed_matrix<T, A> const &m) {
  const void *rp = dev<unsigned int>(m.handle1()), *ci = dev<unsigned int>(m.handle2()),
             *v = dev<T>(m.handle());
  return cached(Context::Key(VCLGB_CSR, rp, ci, v, m.size1(), m.size2(), m.nnz()),
                [&](vclgbBackend be) {
                  vclgbMatrix h = nullptr;
                  check(vclgbCsrCreate(be, prec<T>(), (uint32_t)m.size1(), (uint32_t)m.size2(),
                                       (uint32_t)m.nnz(), static_cast<const uint32_t *>(rp),
                                       static_cast<const uint32_t *>(ci), v, &h),
                        "compressed_matrix");
                  return h;
                });
}

template <typename T>
inline vclgbMatrix handle_of(viennacl::ell_matrix<T, 1> const &m) {
  const void *co = dev<unsigned int>(m.handle2()), *el = dev<T>(m.handle());
  return cached(Context::Key(VCLGB_ELL, co, el, nullptr, m.size1(), m.size2(), m.internal_maxnnz()),
                [&](vclgbBackend be) {
                  vclgbMatrix h = nullptr;
                  check(vclgbEllWrap(be, prec<T>(), (uint32_t)m.size1(), (uint32_t)m.size2(),
                                     (uint32_t)m.internal_maxnnz(),
                                     static_cast<const uint32_t *>(co), el, &h),
                        "ell_matrix");
                  return h;
                });
}

template <typename T>
inline vclgbMatrix handle_of(viennacl::sliced_ell_matrix<T, unsigned int> const &m) {
  const void *cpb = dev<unsigned int>(m.handle1()), *ci = dev<unsigned int>(m.handle2()),
             *bs = dev<unsigned int>(m.handle3()), *el = dev<T>(m.handle());
  return cached(Context::Key(VCLGB_SELL, cpb, ci, el, m.size1(), m.size2(), m.rows_per_block()),
                [&](vclgbBackend be) {
                  vclgbMatrix h = nullptr;
                  check(vclgbSellWrap(be, prec<T>(), (uint32_t)m.size1(), (uint32_t)m.size2(),
                                      (uint32_t)m.rows_per_block(),
                                      static_cast<const uint32_t *>(cpb),
                                      static_cast<const uint32_t *>(ci),
                                      static_cast<const uint32_t *>(bs), el, &h),
                        "sliced_ell_matrix");
                  return h;
                });
}

template <typename T>
inline vclgbMatrix handle_of(viennacl::hyb_matrix<T, 1> const &m) {
  const void *co = dev<unsigned int>(m.handle2()), *el = dev<T>(m.handle());
  const void *trp = dev<unsigned int>(m.handle3());
  return cached(Context::Key(VCLGB_HYB, co, el, trp, m.size1(), m.size2(), m.internal_ellnnz()),
                [&](vclgbBackend be) {
                  // the tail's entry count is its last row pointer (csr_nnz()
                  // counts the placeholder entry of an empty tail)
                  uint32_t tnnz = 0;
                  if (cudaMemcpy(&tnnz, static_cast<const uint32_t *>(trp) + m.size1(), 4,
                                 cudaMemcpyDeviceToHost) != cudaSuccess)
                    throw std::runtime_error("vclgb: hyb_matrix tail size");
                  vclgbMatrix h = nullptr;
                  check(vclgbHybWrap(be, prec<T>(), (uint32_t)m.size1(), (uint32_t)m.size2(),
                                     (uint32_t)m.internal_ellnnz(),
                                     static_cast<const uint32_t *>(co), el,
                                     static_cast<const uint32_t *>(trp),
                                     static_cast<const uint32_t *>(dev<unsigned int>(m.handle4())),
                                     dev<T>(m.handle5()), tnnz, &h),
                        "hyb_matrix");
                  return h;
                });
}

template <typename T>
inline vclgbMatrix handle_of(viennacl::coordinate_matrix<T, 128> const &m) {
  const void *co = dev<unsigned int>(m.handle12()), *el = dev<T>(m.handle());
  return cached(Context::Key(VCLGB_COO, co, el, nullptr, m.size1(), m.size2(), m.nnz()),
                [&](vclgbBackend be) {
                  vclgbMatrix h = nullptr;
                  check(vclgbCooWrap(be, prec<T>(), (uint32_t)m.size1(), (uint32_t)m.size2(),
                                     m.nnz(), static_cast<const uint32_t *>(co), el, &h),
                        "coordinate_matrix");
                  return h;
                });
}

// y = alpha*A*x + beta*y with the vectors' start and stride
template <typename T, typename M>
inline void spmv(M const &mat, viennacl::vector_base<T> const &x, T alpha,
                 viennacl::vector_base<T> &y, T beta) {
  vclgbMatrix h = handle_of(mat);
  check(vclgbSpmv(ctx().be, h, (double)alpha, viennacl::cuda_arg(x), (int64_t)x.start(),
                  (int64_t)x.stride(), (double)beta, viennacl::cuda_arg(y), (int64_t)y.start(),
                  (int64_t)y.stride()),
        "prod");
  // ViennaCL's kernels that follow run on the legacy default stream, which the
  // backend's blocking stream is ordered with
}

template <typename T, typename M>
inline void tri_solve(M const &mat, viennacl::vector_base<T> &vec, int tag, int trans) {
  if (vec.start() != 0 || vec.stride() != 1)
    throw std::runtime_error("vclgb: inplace_solve needs a contiguous vector");
  check(vclgbCsrInplaceSolve(ctx().be, handle_of(mat), tag, trans, viennacl::cuda_arg(vec)),
        "inplace_solve");
}

}  // namespace vclgb_viennacl

namespace viennacl {
namespace linalg {
namespace cuda {

// Templates more specialised than the reference's (alignment 1, unsigned
// indices, COO alignment 128), so partial ordering picks them; as templates
// they need the matrix types complete only where a program uses them.
template <typename NumericT>
inline void prod_impl(const viennacl::compressed_matrix<NumericT, 1> &mat,
                      const viennacl::vector_base<NumericT> &vec, NumericT alpha,
                      viennacl::vector_base<NumericT> &result, NumericT beta) {
  vclgb_viennacl::spmv<NumericT>(mat, vec, alpha, result, beta);
}
template <typename NumericT>
inline void prod_impl(const viennacl::ell_matrix<NumericT, 1> &mat,
                      const viennacl::vector_base<NumericT> &vec, NumericT alpha,
                      viennacl::vector_base<NumericT> &result, NumericT beta) {
  vclgb_viennacl::spmv<NumericT>(mat, vec, alpha, result, beta);
}
template <typename NumericT>
inline void prod_impl(const viennacl::hyb_matrix<NumericT, 1> &mat,
                      const viennacl::vector_base<NumericT> &vec, NumericT alpha,
                      viennacl::vector_base<NumericT> &result, NumericT beta) {
  vclgb_viennacl::spmv<NumericT>(mat, vec, alpha, result, beta);
}
template <typename NumericT>
inline void prod_impl(const viennacl::sliced_ell_matrix<NumericT, unsigned int> &mat,
                      const viennacl::vector_base<NumericT> &vec, NumericT alpha,
                      viennacl::vector_base<NumericT> &result, NumericT beta) {
  vclgb_viennacl::spmv<NumericT>(mat, vec, alpha, result, beta);
}
template <typename NumericT>
inline void prod_impl(const viennacl::coordinate_matrix<NumericT, 128> &mat,
                      const viennacl::vector_base<NumericT> &vec, NumericT alpha,
                      viennacl::vector_base<NumericT> &result, NumericT beta) {
  vclgb_viennacl::spmv<NumericT>(mat, vec, alpha, result, beta);
}

// inplace_solve(A, vec, tag) / inplace_solve(trans(A), vec, tag)
#define VCLGB_SHADOW_TRI(TAG, CODE)                                                         \
  template <typename NumericT>                                                              \
  inline void inplace_solve(const viennacl::compressed_matrix<NumericT, 1> &mat,            \
                            viennacl::vector_base<NumericT> &vec, viennacl::linalg::TAG) {  \
    vclgb_viennacl::tri_solve<NumericT>(mat, vec, CODE, 0);                                 \
  }                                                                                         \
  template <typename NumericT>                                                              \
  inline void inplace_solve(                                                                \
      const matrix_expression<const viennacl::compressed_matrix<NumericT, 1>,               \
                              const viennacl::compressed_matrix<NumericT, 1>, op_trans> &mat, \
      viennacl::vector_base<NumericT> &vec, viennacl::linalg::TAG) {                        \
    vclgb_viennacl::tri_solve<NumericT>(mat.lhs(), vec, CODE, 1);                           \
  }
VCLGB_SHADOW_TRI(lower_tag, VCLGB_LOWER)
VCLGB_SHADOW_TRI(upper_tag, VCLGB_UPPER)
VCLGB_SHADOW_TRI(unit_lower_tag, VCLGB_UNIT_LOWER)
VCLGB_SHADOW_TRI(unit_upper_tag, VCLGB_UNIT_UPPER)
#undef VCLGB_SHADOW_TRI

}  // namespace cuda
}  // namespace linalg
}  // namespace viennacl

#endif
