// blas1.cu -- inner_prod / norm_2 with the result left in device memory.
// The reference reduces to 128 block partials and then either runs a second
// one-block kernel or copies the partials to the host
// (linalg/cuda/vector_operations.hpp:1272-1585, 2017-2448); here one kernel
// does both stages (last-block-done, fixed summation order).
#include "formats.hpp"
#include "vecpass.cuh"

namespace vclgb {

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

}  // namespace vclgb
