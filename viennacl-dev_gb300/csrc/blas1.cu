// blas1.cu -- inner_prod / norm_2 with the result left in device memory.
// The reference reduces to 128 block partials and then either runs a second
// one-block kernel or copies the partials to the host
// (linalg/cuda/vector_operations.hpp:1272-1585, 2017-2448); here one kernel
// does both stages (last-block-done, fixed summation order).
#include <type_traits>
#include <utility>

#include "formats.hpp"
#include "vecpass.cuh"

namespace vclgb {

struct NoScalV {};

template <typename T>
struct DotF {
  static constexpr int NDOT = 1;
  const T *x; int64_t xs, xi;
  const T *y; int64_t ys, yi;
  T *out; bool sq;
  __device__ bool skip() const { return false; }
  struct S {};
  __device__ S load() const { return {}; }
  __device__ void apply(size_t i, S, T (&d)[1]) const {
    d[0] += x[xs + (int64_t)i * xi] * y[ys + (int64_t)i * yi];
  }
  __device__ void finalize(const T (&s)[1]) const { *out = sq ? sqrt(s[0]) : s[0]; }
};

void dot_launch(Backend &be, vclgbPrecision prec, uint64_t n, const void *x, int64_t xs,
                int64_t xinc, const void *y, int64_t ys, int64_t yinc, void *d_result,
                bool sqrt_result) {
  Reduction red{be.red_partials.ptr, be.red_counter.as<unsigned>()};
  if (n == 0) {
    VCLGB_CUDA(cudaMemsetAsync(d_result, 0, prec == VCLGB_FLOAT64 ? 8 : 4, be.stream));
    return;
  }
  if (prec == VCLGB_FLOAT64)
    vec_pass<double>(be, n,
                     DotF<double>{static_cast<const double *>(x), xs, xinc,
                                  static_cast<const double *>(y), ys, yinc,
                                  static_cast<double *>(d_result), sqrt_result},
                     red);
  else
    vec_pass<float>(be, n,
                    DotF<float>{static_cast<const float *>(x), xs, xinc,
                                static_cast<const float *>(y), ys, yinc,
                                static_cast<float *>(d_result), sqrt_result},
                    red);
}


// ---------------------------------------------------------------------------
// Vector updates and element-wise operations (linalg/vector_operations.hpp
// av :78-105, avbv :107-142, avbv_v :144-183, vector_assign :187-216,
// vector_swap :218-250, element_op :255-345; CUDA backend
// linalg/cuda/vector_operations.hpp:77-760, 870-1245).  One grid-stride pass
// each (the vector-pass kernel without a reduction); strided operands.  The
// products, quotients and sums are separately rounded (__dmul_rn, __dadd_rn,
// ...), as the reference's expressions are evaluated, so av/avbv/avbv_v and
// element_prod/element_div are bit-identical to a host evaluation of the same
// expressions; pow and the unary functions call CUDA's math library.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

template <typename T>
struct Strided {
  T *p;
  int64_t s, inc;
  __device__ __forceinline__ T &operator[](size_t i) const { return p[s + (int64_t)i * inc]; }
};

// a scalar operand: a device value (d != nullptr) or a host value, negated
// first when flip is set (the flip_sign argument of av/avbv)
template <typename T>
struct ScalarOp {
  T h;
  const T *d;
  int flip;
  __device__ __forceinline__ T get() const {
    const T a = d ? *d : h;
    return flip ? -a : a;
  }
};

// y = x op a [+ z op b], or y += ... (ACC); op is * or / (RA, RB)
template <typename T, bool RA, bool RB, bool HASZ, bool ACC>
struct AvbvF {
  static constexpr int NDOT = 0;
  Strided<T> y, x, z;
  ScalarOp<T> a, b;
  struct S { T a, b; };
  __device__ bool skip() const { return false; }
  __device__ S load() const { return {a.get(), HASZ ? b.get() : T(0)}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const {
    T t = RA ? div_rn(x[i], c.a) : mul_rn(x[i], c.a);
    if constexpr (HASZ) t = add_rn(t, RB ? div_rn(z[i], c.b) : mul_rn(z[i], c.b));
    if constexpr (ACC) t = add_rn(y[i], t);
    y[i] = t;
  }
  __device__ void finalize(const T (&)[1]) const {}
};

// y = x OP z with either operand possibly a scalar
template <typename T, int OP, bool XS, bool ZS>
struct BinaryF {
  static constexpr int NDOT = 0;
  Strided<T> y, x, z;
  ScalarOp<T> xs, zs;
  struct S { T x, z; };
  __device__ bool skip() const { return false; }
  __device__ S load() const { return {XS ? xs.get() : T(0), ZS ? zs.get() : T(0)}; }
  __device__ void apply(size_t i, S c, T (&)[1]) const {
    const T u = XS ? c.x : x[i], v = ZS ? c.z : z[i];
    if constexpr (OP == VCLGB_OP_PROD) y[i] = mul_rn(u, v);
    else if constexpr (OP == VCLGB_OP_DIV) y[i] = div_rn(u, v);
    else y[i] = pow(u, v);
  }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T, int OP>
__device__ __forceinline__ T unary_apply(T v) {
  switch (OP) {
    case VCLGB_OP_ABS: return abs(v);
    case VCLGB_OP_ACOS: return acos(v);
    case VCLGB_OP_ACOSH: return acosh(v);
    case VCLGB_OP_ASIN: return asin(v);
    case VCLGB_OP_ASINH: return asinh(v);
    case VCLGB_OP_ATAN: return atan(v);
    case VCLGB_OP_ATANH: return atanh(v);
    case VCLGB_OP_CEIL: return ceil(v);
    case VCLGB_OP_COS: return cos(v);
    case VCLGB_OP_COSH: return cosh(v);
    case VCLGB_OP_ERF: return erf(v);
    case VCLGB_OP_ERFC: return erfc(v);
    case VCLGB_OP_EXP: return exp(v);
    case VCLGB_OP_EXP2: return exp2(v);
    // op_exp10 is exp(x * ln 10) in the reference (linalg/detail/op_applier.hpp)
    case VCLGB_OP_EXP10: return exp(mul_rn(v, T(2.302585092994045684017991454684364207601101488628772976033)));
    case VCLGB_OP_FABS: return fabs(v);
    case VCLGB_OP_FLOOR: return floor(v);
    case VCLGB_OP_LOG: return log(v);
    case VCLGB_OP_LOG2: return log2(v);
    case VCLGB_OP_LOG10: return log10(v);
    case VCLGB_OP_ROUND: return round(v);
    case VCLGB_OP_SIN: return sin(v);
    case VCLGB_OP_SINH: return sinh(v);
    case VCLGB_OP_SQRT: return sqrt(v);
    case VCLGB_OP_TAN: return tan(v);
    case VCLGB_OP_TANH: return tanh(v);
    case VCLGB_OP_TRUNC: return trunc(v);
    case VCLGB_OP_RSQRT: return pow(v, T(-0.5));  // pow(x, -0.5) as the reference
    default: return v > T(0) ? T(1) : (v < T(0) ? T(-1) : T(0));  // sign
  }
}

template <typename T, int OP>
struct UnaryF {
  static constexpr int NDOT = 0;
  Strided<T> y, x;
  __device__ bool skip() const { return false; }
  __device__ NoScalV load() const { return {}; }
  __device__ void apply(size_t i, NoScalV, T (&)[1]) const { y[i] = unary_apply<T, OP>(x[i]); }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
struct AssignF {
  static constexpr int NDOT = 0;
  Strided<T> y;
  T a;
  __device__ bool skip() const { return false; }
  __device__ NoScalV load() const { return {}; }
  __device__ void apply(size_t i, NoScalV, T (&)[1]) const { y[i] = a; }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
struct SwapF {
  static constexpr int NDOT = 0;
  Strided<T> x, y;
  __device__ bool skip() const { return false; }
  __device__ NoScalV load() const { return {}; }
  __device__ void apply(size_t i, NoScalV, T (&)[1]) const {
    const T t = x[i];
    x[i] = y[i];
    y[i] = t;
  }
  __device__ void finalize(const T (&)[1]) const {}
};

template <typename T>
static void avbv_t(Backend &be, uint64_t n, const VecArg &y, const VecArg &x,
                   const vclgbScalarArg &a, const VecArg *z, const vclgbScalarArg *b, bool acc) {
  Reduction red{be.red_partials.ptr, be.red_counter.as<unsigned>()};
  auto sv = [](const VecArg &v) { return Strided<T>{static_cast<T *>(const_cast<void *>(v.p)), v.start, v.stride}; };
  auto so = [](const vclgbScalarArg &s) {
    return ScalarOp<T>{static_cast<T>(s.value), static_cast<const T *>(s.d_value), s.flip_sign};
  };
  const Strided<T> sy = sv(y), sx = sv(x), sz = z ? sv(*z) : Strided<T>{nullptr, 0, 1};
  const ScalarOp<T> oa = so(a), ob = b ? so(*b) : ScalarOp<T>{T(0), nullptr, 0};
  // every combination of the four flags is its own kernel (no per-element branch)
  auto go = [&](auto ra, auto rb, auto hz, auto ac) {
    vec_pass<T>(be, n,
                AvbvF<T, decltype(ra)::value, decltype(rb)::value, decltype(hz)::value,
                      decltype(ac)::value>{sy, sx, sz, oa, ob},
                red);
  };
  using F = std::false_type;
  using Tr = std::true_type;
  auto g3 = [&](auto ra, auto rb, auto hz) { acc ? go(ra, rb, hz, Tr{}) : go(ra, rb, hz, F{}); };
  auto g2 = [&](auto ra, auto rb) { z ? g3(ra, rb, Tr{}) : g3(ra, rb, F{}); };
  auto g1 = [&](auto ra) { (b && b->reciprocal) ? g2(ra, Tr{}) : g2(ra, F{}); };
  a.reciprocal ? g1(Tr{}) : g1(F{});
}

void avbv(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y, const VecArg &x,
          const vclgbScalarArg &a, const VecArg *z, const vclgbScalarArg *b, bool acc) {
  if (n == 0) return;
  if (prec == VCLGB_FLOAT64) avbv_t<double>(be, n, y, x, a, z, b, acc);
  else avbv_t<float>(be, n, y, x, a, z, b, acc);
}

template <typename T, int OP>
static void binary_t(Backend &be, uint64_t n, const VecArg &y, const VecArg *x,
                     const vclgbScalarArg &xs, const VecArg *z, const vclgbScalarArg &zs) {
  Reduction red{be.red_partials.ptr, be.red_counter.as<unsigned>()};
  auto sv = [](const VecArg *v) {
    return v ? Strided<T>{static_cast<T *>(const_cast<void *>(v->p)), v->start, v->stride}
             : Strided<T>{nullptr, 0, 1};
  };
  const ScalarOp<T> ox{static_cast<T>(xs.value), static_cast<const T *>(xs.d_value), xs.flip_sign};
  const ScalarOp<T> oz{static_cast<T>(zs.value), static_cast<const T *>(zs.d_value), zs.flip_sign};
  const Strided<T> sy = sv(&y);
  if (x && z) vec_pass<T>(be, n, BinaryF<T, OP, false, false>{sy, sv(x), sv(z), ox, oz}, red);
  else if (z) vec_pass<T>(be, n, BinaryF<T, OP, true, false>{sy, sv(x), sv(z), ox, oz}, red);
  else if (x) vec_pass<T>(be, n, BinaryF<T, OP, false, true>{sy, sv(x), sv(z), ox, oz}, red);
  else throw Error(VCLGB_INVALID_ARGUMENT, "element_op needs at least one vector operand");
}

void element_binary(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y,
                    const VecArg *x, const vclgbScalarArg &xs, const VecArg *z,
                    const vclgbScalarArg &zs, int op) {
  if (n == 0) return;
  require(op >= VCLGB_OP_PROD && op <= VCLGB_OP_POW, VCLGB_INVALID_ARGUMENT,
          "binary op must be VCLGB_OP_PROD, VCLGB_OP_DIV or VCLGB_OP_POW");
  auto run = [&](auto t) {
    using T = decltype(t);
    if (op == VCLGB_OP_PROD) binary_t<T, VCLGB_OP_PROD>(be, n, y, x, xs, z, zs);
    else if (op == VCLGB_OP_DIV) binary_t<T, VCLGB_OP_DIV>(be, n, y, x, xs, z, zs);
    else binary_t<T, VCLGB_OP_POW>(be, n, y, x, xs, z, zs);
  };
  if (prec == VCLGB_FLOAT64) run(double{});
  else run(float{});
}

template <typename T, int OP>
static void unary_one(Backend &be, uint64_t n, const VecArg &y, const VecArg &x) {
  Reduction red{be.red_partials.ptr, be.red_counter.as<unsigned>()};
  vec_pass<T>(be, n,
              UnaryF<T, OP>{Strided<T>{static_cast<T *>(const_cast<void *>(y.p)), y.start, y.stride},
                            Strided<T>{static_cast<T *>(const_cast<void *>(x.p)), x.start, x.stride}},
              red);
}

template <typename T, int... OPS>
static void unary_dispatch(Backend &be, uint64_t n, const VecArg &y, const VecArg &x, int op,
                           std::integer_sequence<int, OPS...>) {
  bool done = false;
  ((op == OPS ? (unary_one<T, OPS>(be, n, y, x), done = true) : false), ...);
  require(done, VCLGB_INVALID_ARGUMENT, "unknown unary element operation");
}

template <int... I>
static std::integer_sequence<int, (I + VCLGB_OP_ABS)...> shift_seq(std::integer_sequence<int, I...>) {
  return {};
}

void element_unary(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y,
                   const VecArg &x, int op) {
  if (n == 0) return;
  const auto ops = shift_seq(std::make_integer_sequence<int, VCLGB_OP_SIGN - VCLGB_OP_ABS + 1>{});
  if (prec == VCLGB_FLOAT64) unary_dispatch<double>(be, n, y, x, op, ops);
  else unary_dispatch<float>(be, n, y, x, op, ops);
}

void vector_assign(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y, double a) {
  if (n == 0) return;
  Reduction red{be.red_partials.ptr, be.red_counter.as<unsigned>()};
  if (prec == VCLGB_FLOAT64)
    vec_pass<double>(be, n, AssignF<double>{{static_cast<double *>(const_cast<void *>(y.p)), y.start, y.stride}, a}, red);
  else
    vec_pass<float>(be, n, AssignF<float>{{static_cast<float *>(const_cast<void *>(y.p)), y.start, y.stride}, (float)a}, red);
}

void vector_swap(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &x, const VecArg &y) {
  if (n == 0) return;
  Reduction red{be.red_partials.ptr, be.red_counter.as<unsigned>()};
  if (prec == VCLGB_FLOAT64)
    vec_pass<double>(be, n, SwapF<double>{{static_cast<double *>(const_cast<void *>(x.p)), x.start, x.stride},
                                          {static_cast<double *>(const_cast<void *>(y.p)), y.start, y.stride}}, red);
  else
    vec_pass<float>(be, n, SwapF<float>{{static_cast<float *>(const_cast<void *>(x.p)), x.start, x.stride},
                                        {static_cast<float *>(const_cast<void *>(y.p)), y.start, y.stride}}, red);
}

}  // namespace vclgb
