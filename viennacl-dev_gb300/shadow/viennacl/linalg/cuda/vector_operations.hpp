// Stands in for ViennaCL's viennacl/linalg/cuda/vector_operations.hpp: includes
// the original, then routes to the engine's C ABI, for float and double:
//   av / avbv / avbv_v (original :144-760) with host or device (viennacl::scalar)
//   scalars, element_op for element_prod / element_div (:1048-1245),
//   inner_prod_impl / inner_prod_cpu (:1519-1580) and norm_2_impl / norm_2_cpu
//   (:2412-2448).
// The reference's dispatcher (viennacl/linalg/vector_operations.hpp:78-345,
// 497-790) calls these overloads, which as exact non-template matches win over
// its templates.
#ifndef VCLGB_SHADOW_CUDA_VECTOR_OPERATIONS_HPP
#define VCLGB_SHADOW_CUDA_VECTOR_OPERATIONS_HPP

#include_next <viennacl/linalg/cuda/vector_operations.hpp>

#include <cuda_runtime.h>

#include "vclgb_viennacl.hpp"

namespace vclgb_viennacl {

template <typename T>
inline vclgbScalarArg sarg(T const &a, bool reciprocal, bool flip) {
  vclgbScalarArg s;
  s.value = (double)a;
  s.d_value = nullptr;
  s.reciprocal = reciprocal;
  s.flip_sign = flip;
  return s;
}
template <typename T>
inline vclgbScalarArg sarg(viennacl::scalar<T> const &a, bool reciprocal, bool flip) {
  vclgbScalarArg s;
  s.value = 0.0;
  s.d_value = viennacl::cuda_arg(a);
  s.reciprocal = reciprocal;
  s.flip_sign = flip;
  return s;
}

template <typename T, typename SA, typename SB>
inline void avbv(viennacl::vector_base<T> &v1, viennacl::vector_base<T> const &v2, SA const &a,
                 bool ra, bool fa, viennacl::vector_base<T> const *v3, SB const *b, bool rb,
                 bool fb, int acc) {
  vclgbScalarArg sb = b ? sarg(*b, rb, fb) : sarg(T(0), false, false);
  check(vclgbAvbv(ctx().be, prec<T>(), v1.size(), viennacl::cuda_arg(v1), (int64_t)v1.start(),
                  (int64_t)v1.stride(), viennacl::cuda_arg(v2), (int64_t)v2.start(),
                  (int64_t)v2.stride(), sarg(a, ra, fa), v3 ? viennacl::cuda_arg(*v3) : nullptr,
                  v3 ? (int64_t)v3->start() : 0, v3 ? (int64_t)v3->stride() : 1, sb, acc),
        "vector update");
}

template <typename T>
inline void binary(viennacl::vector_base<T> &v1, viennacl::vector_base<T> const &v2,
                   viennacl::vector_base<T> const &v3, int op) {
  const vclgbScalarArg none = sarg(T(0), false, false);
  check(vclgbElementBinary(ctx().be, prec<T>(), v1.size(), viennacl::cuda_arg(v1),
                           (int64_t)v1.start(), (int64_t)v1.stride(), viennacl::cuda_arg(v2),
                           (int64_t)v2.start(), (int64_t)v2.stride(), none,
                           viennacl::cuda_arg(v3), (int64_t)v3.start(), (int64_t)v3.stride(),
                           none, op),
        "element_op");
}

// the operands of an element-wise expression (a template, so that ViennaCL's
// expression types need only be complete where it is used)
template <typename T, typename E>
inline void binary_expr(viennacl::vector_base<T> &v1, E const &proxy, int op) {
  binary<T>(v1, proxy.lhs(), proxy.rhs(), op);
}

template <typename T, typename S>
inline T *scalar_ptr(S &s) {
  return viennacl::cuda_arg(s);
}

template <typename T>
inline void dot(viennacl::vector_base<T> const &v1, viennacl::vector_base<T> const &v2,
                T *d_result) {
  check(vclgbDot(ctx().be, prec<T>(), v1.size(), viennacl::cuda_arg(v1), (int64_t)v1.start(),
                 (int64_t)v1.stride(), viennacl::cuda_arg(v2), (int64_t)v2.start(),
                 (int64_t)v2.stride(), d_result),
        "inner_prod");
}

template <typename T>
inline void nrm2(viennacl::vector_base<T> const &v, T *d_result) {
  check(vclgbNorm2(ctx().be, prec<T>(), v.size(), viennacl::cuda_arg(v), (int64_t)v.start(),
                   (int64_t)v.stride(), d_result),
        "norm_2");
}

// a device scalar's value on the host (the reference's *_cpu variants)
template <typename T, typename F>
inline void to_host(T &out, F &&compute) {
  T *d = nullptr;
  if (cudaMalloc(&d, sizeof(T)) != cudaSuccess) throw std::runtime_error("vclgb: scalar");
  compute(d);
  check(vclgbBackendSynchronize(ctx().be), "synchronize");
  cudaMemcpy(&out, d, sizeof(T), cudaMemcpyDeviceToHost);
  cudaFree(d);
}

}  // namespace vclgb_viennacl

namespace viennacl {
namespace linalg {
namespace cuda {

#define VCLGB_SHADOW_VECOPS(T)                                                                    \
  inline void av(vector_base<T> &v1, vector_base<T> const &v2, T const &a, vcl_size_t, bool ra,  \
                 bool fa) {                                                                       \
    vclgb_viennacl::avbv<T, T, T>(v1, v2, a, ra, fa, nullptr, nullptr, false, false, 0);         \
  }                                                                                               \
  inline void av(vector_base<T> &v1, vector_base<T> const &v2, viennacl::scalar<T> const &a,     \
                 vcl_size_t, bool ra, bool fa) {                                                  \
    vclgb_viennacl::avbv<T, viennacl::scalar<T>, T>(v1, v2, a, ra, fa, nullptr, nullptr, false,  \
                                                    false, 0);                                    \
  }                                                                                               \
  VCLGB_SHADOW_AVBV(T, T, T)                                                                      \
  VCLGB_SHADOW_AVBV(T, T, viennacl::scalar<T>)                                                    \
  VCLGB_SHADOW_AVBV(T, viennacl::scalar<T>, T)                                                    \
  VCLGB_SHADOW_AVBV(T, viennacl::scalar<T>, viennacl::scalar<T>)                                  \
  inline void element_op(                                                                         \
      vector_base<T> &v1,                                                                         \
      vector_expression<const vector_base<T>, const vector_base<T>, op_element_binary<op_prod> >  \
          const &proxy) {                                                                         \
    vclgb_viennacl::binary_expr<T>(v1, proxy, VCLGB_OP_PROD);                                     \
  }                                                                                               \
  inline void element_op(                                                                         \
      vector_base<T> &v1,                                                                         \
      vector_expression<const vector_base<T>, const vector_base<T>, op_element_binary<op_div> >   \
          const &proxy) {                                                                         \
    vclgb_viennacl::binary_expr<T>(v1, proxy, VCLGB_OP_DIV);                                      \
  }                                                                                               \
  inline void inner_prod_impl(vector_base<T> const &v1, vector_base<T> const &v2,                 \
                              scalar<T> &result) {                                                \
    vclgb_viennacl::dot<T>(v1, v2, vclgb_viennacl::scalar_ptr<T>(result));                        \
  }                                                                                               \
  inline void inner_prod_cpu(vector_base<T> const &v1, vector_base<T> const &v2, T &result) {    \
    vclgb_viennacl::to_host(result, [&](T *d) { vclgb_viennacl::dot<T>(v1, v2, d); });           \
  }                                                                                               \
  inline void norm_2_impl(vector_base<T> const &v, scalar<T> &result) {                           \
    vclgb_viennacl::nrm2<T>(v, vclgb_viennacl::scalar_ptr<T>(result));                            \
  }                                                                                               \
  inline void norm_2_cpu(vector_base<T> const &v, T &result) {                                    \
    vclgb_viennacl::to_host(result, [&](T *d) { vclgb_viennacl::nrm2<T>(v, d); });               \
  }

#define VCLGB_SHADOW_AVBV(T, SA, SB)                                                              \
  inline void avbv(vector_base<T> &v1, vector_base<T> const &v2, SA const &a, vcl_size_t,         \
                   bool ra, bool fa, vector_base<T> const &v3, SB const &b, vcl_size_t, bool rb,  \
                   bool fb) {                                                                     \
    vclgb_viennacl::avbv<T, SA, SB>(v1, v2, a, ra, fa, &v3, &b, rb, fb, 0);                       \
  }                                                                                               \
  inline void avbv_v(vector_base<T> &v1, vector_base<T> const &v2, SA const &a, vcl_size_t,       \
                     bool ra, bool fa, vector_base<T> const &v3, SB const &b, vcl_size_t,         \
                     bool rb, bool fb) {                                                          \
    vclgb_viennacl::avbv<T, SA, SB>(v1, v2, a, ra, fa, &v3, &b, rb, fb, 1);                       \
  }

VCLGB_SHADOW_VECOPS(double)
VCLGB_SHADOW_VECOPS(float)
#undef VCLGB_SHADOW_VECOPS
#undef VCLGB_SHADOW_AVBV

}  // namespace cuda
}  // namespace linalg
}  // namespace viennacl

#endif
