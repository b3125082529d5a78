// tune.cu -- per-matrix SpMV autotuner (no reference counterpart; the
// reference's sliced_ell_matrix takes its slice height from the caller and has
// no sort window, and its CSR kernel choice is a fixed rule,
// linalg/cuda/sparse_matrix_operations.hpp:262-396).
//
// The candidates are the CSR kernel the row-length analysis picks (its lanes
// per row follow each row's length class), SELL-C-sigma for slice heights C in
// {32, 64} and sort windows sigma in {1, C, 256, 1024, 4096}, HYB (csr_threshold
// 0.8) and ELL where its padding stays below twice the nonzeros.  Each is
// converted on the device and timed over a few products (CUDA events, the
// mean of the launches after one warm-up); forms that pad beyond 8 x nnz are
// skipped.  The fastest form is kept on the matrix (Matrix::tuned) and every
// later product on it -- vclgbSpmv and the solvers' SpMV phases -- runs on
// that form; the tuned form is a converted copy, so a matrix whose values
// change is re-tuned or cleared first.
#include <algorithm>
#include <cmath>

#include "formats.hpp"
#include "spmv.cuh"

namespace vclgb {

template <typename T>
static double time_spmv(Backend &be, const Matrix &m, const T *x, T *y, int reps) {
  Reduction red{be.red_partials.ptr, be.red_counter.as<unsigned>()};
  DevBuf hyb;
  if (hyb_scratch_bytes(m)) hyb.alloc(hyb_scratch_bytes(m), be.stream);
  auto once = [&]() {
    EpiAxpbyM<T, 0, true> e{};
    e.alpha = T(1); e.beta = T(0); e.y = y; e.ys = 0; e.yinc = 1;
    spmv_launch<T>(be, m, x, 0, 1, e, red, y, 0, 1, T(1), T(0), nullptr, hyb.ptr);
  };
  once();  // warm-up (first launches of the instantiation)
  cudaEvent_t e0, e1;
  VCLGB_CUDA(cudaEventCreate(&e0));
  VCLGB_CUDA(cudaEventCreate(&e1));
  VCLGB_CUDA(cudaEventRecord(e0, be.stream));
  for (int i = 0; i < reps; ++i) once();
  VCLGB_CUDA(cudaEventRecord(e1, be.stream));
  VCLGB_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  VCLGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 1e3 * ms / reps;
}

template <typename T>
static void autotune_t(Backend &be, Matrix &A, vclgbTuneInfo *info) {
  const size_t n = A.rows, nc = A.cols;
  DevBuf xb(std::max<size_t>(nc, 1) * sizeof(T), be.stream), yb(std::max<size_t>(n, 1) * sizeof(T), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(xb.ptr, 0, xb.bytes, be.stream));  // x = 0: timing only
  T *x = xb.as<T>(), *y = yb.as<T>();
  const int reps = 10;
  A.tuned.reset();
  const double t_csr = time_spmv<T>(be, A, x, y, reps);
  double best = t_csr;
  std::unique_ptr<Matrix> best_m;
  uint32_t tried = 1;
  auto consider = [&](std::unique_ptr<Matrix> m) {
    if (!m) return;
    const uint64_t stored = m->format == VCLGB_SELL ? m->sell_stored
                          : m->format == VCLGB_ELL  ? (uint64_t)m->ell_width * m->rows
                                                    : (uint64_t)m->ell_width * m->rows + m->tail_nnz;
    ++tried;
    if (stored > 8 * std::max<uint64_t>(A.nnz, 1)) return;
    const double t = time_spmv<T>(be, *m, x, y, reps);
    if (t < best) {
      best = t;
      best_m = std::move(m);
    }
  };
  for (uint32_t C : {32u, 64u}) {
    for (uint32_t sigma : {1u, C, 256u, 1024u, 4096u}) {
      if (sigma != 1 && sigma < C) continue;
      if (sigma > 1 && (size_t)sigma >= 2 * n) continue;
      consider(convert_sell(be, A, C, sigma));
    }
  }
  consider(convert_hyb(be, A, 0.8));
  if ((uint64_t)A.max_row_len * A.rows <= 2 * std::max<uint64_t>(A.nnz, 1))
    consider(convert_ell(be, A));
  std::memset(info, 0, sizeof(*info));
  info->candidates = tried;
  info->us_csr = t_csr;
  info->us_best = best;
  info->format = VCLGB_CSR;
  if (best_m) {
    info->format = best_m->format;
    info->slice_height = best_m->format == VCLGB_SELL ? best_m->C : 0;
    info->sigma = best_m->format == VCLGB_SELL ? best_m->sigma : 0;
    info->csr_threshold = best_m->format == VCLGB_HYB ? 0.8 : 0.0;
    A.tuned = std::move(best_m);
  }
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
}

void matrix_autotune(Backend &be, Matrix &A, vclgbTuneInfo *info) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "the autotuner starts from a CSR matrix");
  require(info != nullptr, VCLGB_INVALID_ARGUMENT, "info is NULL");
  if (A.rows == 0) {
    std::memset(info, 0, sizeof(*info));
    info->format = VCLGB_CSR;
    return;
  }
  if (A.prec == VCLGB_FLOAT64) autotune_t<double>(be, A, info);
  else autotune_t<float>(be, A, info);
}

}  // namespace vclgb
