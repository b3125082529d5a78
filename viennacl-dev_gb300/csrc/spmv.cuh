// spmv.cuh -- SpMV kernels for CSR (single-bin stencil kernel, row-window kernel
// with per-window length classes), ELL, SELL-C-sigma
// and HYB (ELL + COO tail with a warp-segmented reduction).
//
// Every kernel hands each finished row to an epilogue object E:
//   static constexpr int NDOT;                    number of fused dot products
//   bool skip() const;                            grid-uniform early exit
//   Pre pre(uint32_t r) const;                    per-row operands of the
//                                                 epilogue (y, p, b, diag ...),
//                                                 loaded before the row's
//                                                 products so the loads overlap
//   void row(uint32_t r, T acc, const Pre &, T (&dots)[..])
//                                                 store the row, add to dots
//   void finalize(const T (&sums)[..]) const;     last block, thread 0
// so the pipelined solvers fuse "Ap = A p" with their reductions, as the
// reference's pipelined_*_prod kernels do (linalg/cuda/iterative_operations.hpp),
// but finish the reduction and the scalar recurrences on the device.
#pragma once

#include "vclgb_internal.hpp"

namespace vclgb {

constexpr int kSpmvThreads = 256;

#define VCLGB_NO_PRE                                                    \
  struct Pre {};                                                        \
  __device__ __forceinline__ Pre pre(uint32_t) const { return {}; }

// GB300 executes FP64 arithmetic at a small fraction of its FP32 rate, and an
// FP64 SpMV keeps that pipe busy with its one FMA per entry.  Everything else
// a kernel does per row or per entry is therefore kept off the FP64 pipe:
// the alpha/beta cases are resolved on the host (MODE), and padding zeros are
// recognised by an integer test of the value's bits.
__device__ __forceinline__ bool nonzero_bits(double v) {
  return (__double_as_longlong(v) << 1) != 0;  // +0.0 and -0.0 are zero
}
__device__ __forceinline__ bool nonzero_bits(float v) { return (__float_as_int(v) << 1) != 0; }

// epilogue: y = alpha*acc + beta*y (linalg/cuda/sparse_matrix_operations.hpp prod_impl).
// MODE 0: alpha == 1, beta == 0; MODE 1: beta == 0; MODE 2: general (y read).
// UNIT: y is contiguous (start 0, stride 1), so a row's slot needs no 64-bit
// index arithmetic -- measurable in the padded formats' short per-row paths.
template <typename T, int MODE, bool UNIT = false>
struct EpiAxpbyM {
  static constexpr int NDOT = 0;
  T alpha, beta;
  T *y;
  int64_t ys, yinc;
  struct Pre { T yold; };
  __device__ __forceinline__ T *slot(uint32_t r) const {
    if constexpr (UNIT) return y + r;
    else return y + ys + (int64_t)r * yinc;
  }
  __device__ __forceinline__ bool skip() const { return false; }
  __device__ __forceinline__ Pre pre(uint32_t r) const {
    if constexpr (MODE == 2) return {*slot(r)};
    else return {T(0)};
  }
  __device__ __forceinline__ void row(uint32_t r, T acc, const Pre &pv, T (&)[1]) const {
    T out;
    if constexpr (MODE == 0) out = acc;
    else if constexpr (MODE == 1) out = alpha * acc;
    else out = alpha * acc + beta * pv.yold;
    *slot(r) = out;
  }
  __device__ __forceinline__ void finalize(const T (&)[1]) const {}
};
template <typename T>
using EpiAxpby = EpiAxpbyM<T, 2>;

// calls f(std::integral_constant<int, MODE>) for the alpha/beta case at hand
template <typename T, class F>
void with_axpby_mode(T alpha, T beta, F &&f) {
  if (beta != T(0)) f(std::integral_constant<int, 2>{});
  else if (alpha != T(1)) f(std::integral_constant<int, 1>{});
  else f(std::integral_constant<int, 0>{});
}

// same, with an early-exit flag (solver converged)
template <typename T, int MODE, bool UNIT = false>
struct EpiAxpbySkip : EpiAxpbyM<T, MODE, UNIT> {
  const int *flag;
  __device__ __forceinline__ bool skip() const { return flag && *flag; }
};

template <int N>
struct DotArr { static constexpr int n = N > 0 ? N : 1; };

// ---------------------------------------------------------------------------
// CSR
// ---------------------------------------------------------------------------
template <typename T>
struct CsrView {
  const uint32_t *rp;
  const uint32_t *ci;
  const T *v;
  uint32_t rows;
};

// Rows of one bin, LANES threads per row.  Each lane takes up to MPL entries
// of its row per round (lane, lane+LANES, ...) and issues every value, index
// and x load of the round before the first multiply, so a warp keeps
// 2*MPL*32 independent loads in flight.  For rows of at most 8 entries
// (stencils) LANES = 1: one thread per row, no shuffles.  The warp's groups
// take consecutive rows, so the warp reads one contiguous stretch of the
// value and index arrays.  A slot past the row's end is predicated off but
// its FMA still takes an FP64 issue slot, so a stencil matrix whose longest
// row has 3..7 entries runs with MPL equal to that length.
constexpr int kMpl = 8;

// The warps numbered warp, warp + nwarps, ... share the rows (grid-wide or
// within one block); list may live in global or shared memory.
template <int LANES, int MPL, typename T, class E>
__device__ __forceinline__ void csr_rows_group(const CsrView<T> &A, const T *__restrict__ x,
                                               int64_t xs, int64_t xinc, uint32_t count,
                                               const uint32_t *list, const E &epi,
                                               T (&dots)[DotArr<E::NDOT>::n], size_t warp,
                                               size_t nwarps) {
  constexpr int GPW = 32 / LANES;  // groups per warp
  const uint32_t lane = threadIdx.x & (LANES - 1);
  const uint32_t gw = (threadIdx.x & 31) / LANES;
  for (size_t wb = warp * GPW; wb < count; wb += nwarps * GPW) {
    const size_t idx = wb + gw;
    const bool ok = idx < count;
    const uint32_t row = ok ? (list ? list[idx] : (uint32_t)idx) : 0xffffffffu;
    const uint32_t s = ok ? __ldg(A.rp + row) : 0u;
    const uint32_t e = ok ? __ldg(A.rp + row + 1) : 0u;
    typename E::Pre pv{};
    if (ok && lane == 0) pv = epi.pre(row);
    T acc = T(0);
    for (uint32_t k0 = s + lane; k0 < e; k0 += MPL * LANES) {
      uint32_t c[MPL];
      T vv[MPL];
#pragma unroll
      for (int j = 0; j < MPL; ++j) {
        const uint32_t k = k0 + j * LANES;
        const bool in = k < e;
        c[j] = in ? __ldg(A.ci + k) : 0u;
        vv[j] = in ? __ldg(A.v + k) : T(0);
      }
#pragma unroll
      for (int j = 0; j < MPL; ++j)
        if (k0 + j * LANES < e) acc += vv[j] * __ldg(x + xs + (int64_t)c[j] * xinc);
    }
    if constexpr (LANES > 1) acc = group_sum<LANES>(acc);
    if (lane == 0 && ok) epi.row(row, acc, pv, dots);
  }
}

// Thread per row, two rows per thread and round (rows wb + lane and
// wb + 32 + lane of the warp's 64): two independent FMA chains and twice the
// loads in flight per thread.  Used for the solvers' SpMV phases on stencil
// matrices, whose fused dot products leave the FP64 pipe the binding unit:
// measured on the 128^3 CG phase, 55.2 -> 49.2 us a launch alone at 5 blocks
// of 256 per SM (the registers of the second row), against one row per thread
// at 8 blocks.
template <int MPL, typename T, class E>
__device__ __forceinline__ void csr_rows_pair(const CsrView<T> &A, const T *__restrict__ x,
                                              int64_t xs, int64_t xinc, uint32_t count,
                                              const E &epi, T (&dots)[DotArr<E::NDOT>::n],
                                              size_t warp, size_t nwarps) {
  const uint32_t lane = threadIdx.x & 31;
  for (size_t wb = warp * 64; wb < count; wb += nwarps * 64) {
    uint32_t s[2], e[2];
    typename E::Pre pv[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const size_t row = wb + q * 32 + lane;
      const bool ok = row < count;
      s[q] = ok ? __ldg(A.rp + row) : 0u;
      e[q] = ok ? __ldg(A.rp + row + 1) : 0u;
      pv[q] = typename E::Pre{};
      if (ok) pv[q] = epi.pre((uint32_t)row);
    }
    T acc[2] = {T(0), T(0)};
    uint32_t c[2][MPL];
    T vv[2][MPL];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int j = 0; j < MPL; ++j) {
        const uint32_t k = s[q] + j;
        const bool in = k < e[q];
        c[q][j] = in ? __ldg(A.ci + k) : 0u;
        vv[q][j] = in ? __ldg(A.v + k) : T(0);
      }
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int j = 0; j < MPL; ++j)
        if (s[q] + j < e[q]) acc[q] += vv[q][j] * __ldg(x + xs + (int64_t)c[q][j] * xinc);
    // rows longer than MPL (none in a stencil bin whose MPL is its longest
    // row) finish one at a time
#pragma unroll
    for (int q = 0; q < 2; ++q)
      for (uint32_t k = s[q] + MPL; k < e[q]; ++k)
        acc[q] += __ldg(A.v + k) * __ldg(x + xs + (int64_t)__ldg(A.ci + k) * xinc);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const size_t row = wb + q * 32 + lane;
      if (row < count) epi.row((uint32_t)row, acc[q], pv[q], dots);
    }
  }
}

// one block per row (rows longer than a warp can stream efficiently); the
// block takes rows first, first + step, ... of the list
template <typename T, class E>
__device__ __forceinline__ void csr_rows_block(const CsrView<T> &A, const T *__restrict__ x,
                                               int64_t xs, int64_t xinc, uint32_t count,
                                               const uint32_t *list, const E &epi,
                                               T (&dots)[DotArr<E::NDOT>::n], T *smem,
                                               size_t first, size_t step) {
  for (size_t i = first; i < count; i += step) {
    uint32_t row = list ? list[i] : (uint32_t)i;
    uint32_t s = __ldg(A.rp + row), e = __ldg(A.rp + row + 1);
    typename E::Pre pv{};
    if (threadIdx.x == 0) pv = epi.pre(row);
    T acc[1] = {T(0)};
    for (uint32_t k = s + threadIdx.x; k < e; k += blockDim.x)
      acc[0] += __ldg(A.v + k) * __ldg(x + xs + (int64_t)__ldg(A.ci + k) * xinc);
    block_sum<1>(acc, smem);
    if (threadIdx.x == 0) epi.row(row, acc[0], pv, dots);
    __syncthreads();
  }
}

// Matrices whose rows all fall in one length bin (stencils: longest row at
// most about twice the mean) run without any row classification: LANES
// threads per row, MPL entries per lane and round, rows in order.  PAIR (one
// lane per row, solver phases with fused dots): two rows per thread and
// round, 5 blocks per SM.
template <int LANES, int MPL, typename T, class E, bool PAIR = false>
__global__ void __launch_bounds__(kSpmvThreads,
                                  PAIR ? 5 : ((E::NDOT > 0 && E::NDOT <= 2) ? 8 : 0))
    csr_fixed_kernel(CsrView<T> A, const T *__restrict__ x, int64_t xs, int64_t xinc, E epi,
                     T *partials, unsigned *counter) {
  pdl_trigger();
  pdl_wait();
  if (epi.skip()) return;
  __shared__ T smem[3 * (kSpmvThreads / 32) + 8];
  T dots[DotArr<E::NDOT>::n];
#pragma unroll
  for (int i = 0; i < DotArr<E::NDOT>::n; ++i) dots[i] = T(0);
  const size_t gwarp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t gnwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  if constexpr (PAIR)
    csr_rows_pair<MPL>(A, x, xs, xinc, A.rows, epi, dots, gwarp, gnwarps);
  else
    csr_rows_group<LANES, MPL>(A, x, xs, xinc, A.rows, nullptr, epi, dots, gwarp, gnwarps);
  if constexpr (E::NDOT > 0) {
    T sums[E::NDOT];
    if (grid_reduce<E::NDOT>(dots, partials, counter, smem, sums)) epi.finalize(sums);
  }
}

// ---------------------------------------------------------------------------
// Row-window CSR for irregular row lengths.  A block takes windows of
// kWinRows consecutive rows, sorts the window's rows into length classes in
// shared memory (stable, so the rows a thread handles and the order of its
// dot partials are fixed for a matrix) and runs each class with its own lane
// count.  The values and indices of a window are one contiguous stretch that
// the block reads within a short time, so each sector comes from DRAM once;
// global length bins sweep the whole matrix once per bin and re-read the
// sectors that rows of different bins share.
// ---------------------------------------------------------------------------
constexpr int kWinRounds = 2;                        // rows per thread and window
constexpr int kWinRows = kWinRounds * kSpmvThreads;  // 512
constexpr int kWinClasses = 8;
constexpr int kWinWarps = kSpmvThreads / 32;

// length classes: <=4, <=8 (one lane), <=16 (2), <=32 (4), <=64 (8), <=128 (16),
// <=4096 (32 lanes, rounds of 256 entries), longer (the whole block)
__device__ __forceinline__ uint32_t win_class(uint32_t len) {
  return len <= 4 ? 0u : len <= 8 ? 1u : len <= 16 ? 2u : len <= 32 ? 3u
       : len <= 64 ? 4u : len <= 128 ? 5u : len <= 4096 ? 6u : 7u;
}

template <int LANES, int MPL, typename T, class E>
__device__ __forceinline__ void win_class_rows(const CsrView<T> &A, const T *__restrict__ x,
                                               int64_t xs, int64_t xinc, const uint32_t *lists,
                                               const uint32_t *cstart, int c, uint32_t &slot,
                                               const E &epi, T (&dots)[DotArr<E::NDOT>::n]) {
  constexpr uint32_t GPW = 32 / LANES;
  const uint32_t n = cstart[c + 1] - cstart[c];
  // the class's first rows go to the warp after the last one the previous
  // class used, so small classes do not all land on warp 0
  const uint32_t warp = threadIdx.x >> 5;
  const uint32_t vw = (warp + kWinWarps - slot % kWinWarps) % kWinWarps;
  csr_rows_group<LANES, MPL>(A, x, xs, xinc, n, lists + cstart[c], epi, dots, vw, kWinWarps);
  slot += (n + GPW - 1) / GPW;
}

template <typename T, class E>
__global__ void __launch_bounds__(kSpmvThreads)
    csr_window_kernel(CsrView<T> A, const T *__restrict__ x, int64_t xs, int64_t xinc, E epi,
                      T *partials, unsigned *counter) {
  pdl_trigger();
  pdl_wait();
  if (epi.skip()) return;
  __shared__ T smem[3 * (kSpmvThreads / 32) + 8];
  __shared__ uint32_t lists[kWinRows];
  // rows per (class, round, warp), then their exclusive offsets in lists
  __shared__ uint32_t woff[kWinClasses * kWinRounds * kWinWarps];
  __shared__ uint32_t cstart[kWinClasses + 1];
  T dots[DotArr<E::NDOT>::n];
#pragma unroll
  for (int i = 0; i < DotArr<E::NDOT>::n; ++i) dots[i] = T(0);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t nwin = (A.rows + kWinRows - 1) / kWinRows;
  for (uint32_t w = blockIdx.x; w < nwin; w += gridDim.x) {
    const uint32_t r0 = w * kWinRows;
    uint32_t cls[kWinRounds];
#pragma unroll
    for (int i = 0; i < kWinRounds; ++i) {
      const uint32_t r = r0 + i * kSpmvThreads + threadIdx.x;
      cls[i] = r < A.rows ? win_class(__ldg(A.rp + r + 1) - __ldg(A.rp + r)) : kWinClasses;
#pragma unroll
      for (int c = 0; c < kWinClasses; ++c) {
        const unsigned m = __ballot_sync(0xffffffffu, cls[i] == (uint32_t)c);
        if (lane == 0) woff[(c * kWinRounds + i) * kWinWarps + warp] = __popc(m);
      }
    }
    __syncthreads();
    if (warp == 0) {
      constexpr int N = kWinClasses * kWinRounds * kWinWarps;
      constexpr int PER = N / 32;
      static_assert(N % 32 == 0 && (kWinRounds * kWinWarps) % PER == 0, "window scan layout");
      uint32_t v[PER], t = 0;
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        v[j] = woff[lane * PER + j];
        t += v[j];
      }
      uint32_t incl = t;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t q = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += q;
      }
      uint32_t run = incl - t;
      if ((lane * PER) % (kWinRounds * kWinWarps) == 0)
        cstart[lane * PER / (kWinRounds * kWinWarps)] = run;
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        woff[lane * PER + j] = run;
        run += v[j];
      }
      if (lane == 31) cstart[kWinClasses] = run;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kWinRounds; ++i) {
      const uint32_t c = cls[i];
      const unsigned m = __match_any_sync(0xffffffffu, c);
      if (c < kWinClasses)
        lists[woff[(c * kWinRounds + i) * kWinWarps + warp] + __popc(m & ((1u << lane) - 1u))] =
            r0 + i * kSpmvThreads + threadIdx.x;
    }
    __syncthreads();
    uint32_t slot = 0;
    win_class_rows<1, 4>(A, x, xs, xinc, lists, cstart, 0, slot, epi, dots);
    win_class_rows<1, 8>(A, x, xs, xinc, lists, cstart, 1, slot, epi, dots);
    win_class_rows<2, 8>(A, x, xs, xinc, lists, cstart, 2, slot, epi, dots);
    win_class_rows<4, 8>(A, x, xs, xinc, lists, cstart, 3, slot, epi, dots);
    win_class_rows<8, 8>(A, x, xs, xinc, lists, cstart, 4, slot, epi, dots);
    win_class_rows<16, 8>(A, x, xs, xinc, lists, cstart, 5, slot, epi, dots);
    win_class_rows<32, 8>(A, x, xs, xinc, lists, cstart, 6, slot, epi, dots);
    csr_rows_block(A, x, xs, xinc, cstart[8] - cstart[7], lists + cstart[7], epi, dots, smem, 0, 1);
    __syncthreads();  // lists and cstart are rewritten for the next window
  }
  if constexpr (E::NDOT > 0) {
    T sums[E::NDOT];
    if (grid_reduce<E::NDOT>(dots, partials, counter, smem, sums)) epi.finalize(sums);
  }
}

// ---------------------------------------------------------------------------
// Padded formats (ELL, SELL, the ELL part of HYB) store explicit zeros that the
// reference kernels skip (ELL) or replace by a literal 0 (SELL).  For finite x
// an unconditional FMA of a stored zero adds +-0 and leaves the sum unchanged,
// so the fast path multiplies every slot and issues all x loads up front; a
// value-dependent predicate would make each x load wait for its element load.
// Only a non-finite sum (inf/NaN reached through x) can differ: that row is
// recomputed with stored zeros skipped, the reference result.
// ---------------------------------------------------------------------------
// exponent not all ones (integer test, off the FP64 pipe)
__device__ __forceinline__ bool finite_bits(double v) {
  return (__double2hiint(v) & 0x7ff00000) != 0x7ff00000;
}
__device__ __forceinline__ bool finite_bits(float v) {
  return (__float_as_int(v) & 0x7f800000) != 0x7f800000;
}

// The rare non-finite path: a plain loop (not unrolled), so that it takes no
// registers from the fast path of every row.
template <typename T>
__device__ __forceinline__ T strided_row_skip(size_t base, uint32_t w, size_t stride,
                                           const uint32_t *__restrict__ cols,
                                           const T *__restrict__ elems, const T *__restrict__ x,
                                           int64_t xs, int64_t xinc) {
  T acc = 0;
#pragma unroll 1
  for (uint32_t j = 0; j < w; ++j) {
    const T v = elems[base + (size_t)j * stride];
    if (nonzero_bits(v)) acc += v * x[xs + (int64_t)cols[base + (size_t)j * stride] * xinc];
  }
  return acc;
}

// slots j0 .. j0+R-1 of a row stored at base + j*stride: all R value and
// index loads, then all R x loads, then the R FMAs in slot order
template <int R, typename T>
__device__ __forceinline__ T strided_round(T acc, size_t base, uint32_t j0, size_t stride,
                                           const uint32_t *__restrict__ cols,
                                           const T *__restrict__ elems,
                                           const T *__restrict__ x, int64_t xs, int64_t xinc) {
  T val[R];
  uint32_t col[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const size_t off = base + (size_t)(j0 + q) * stride;
    val[q] = __ldg(elems + off);
    col[q] = __ldg(cols + off);
  }
#pragma unroll
  for (int q = 0; q < R; ++q) acc += val[q] * __ldg(x + xs + (int64_t)col[q] * xinc);
  return acc;
}

// Slots [j0, j1) of a row: full rounds of 8, then one round of exactly the
// remaining count.  No slot is predicated off, so no FMA issue slot is spent
// on padding beyond the stored width (j0 and j1 are warp-uniform in ELL with a
// fixed width and in SELL with C a multiple of 32, so the switch does not
// diverge).
template <typename T>
__device__ __forceinline__ T strided_range(T acc, size_t base, uint32_t j0, uint32_t j1,
                                           size_t stride, const uint32_t *__restrict__ cols,
                                           const T *__restrict__ elems, const T *__restrict__ x,
                                           int64_t xs, int64_t xinc) {
  for (; j0 + 8 <= j1; j0 += 8) acc = strided_round<8>(acc, base, j0, stride, cols, elems, x, xs, xinc);
  switch (j1 - j0) {
#define VCLGB_REM(R) \
  case R: acc = strided_round<R>(acc, base, j0, stride, cols, elems, x, xs, xinc); break;
    VCLGB_REM(1) VCLGB_REM(2) VCLGB_REM(3) VCLGB_REM(4) VCLGB_REM(5) VCLGB_REM(6) VCLGB_REM(7)
#undef VCLGB_REM
    default: break;
  }
  return acc;
}

// a whole row of w slots, with the non-finite fallback
template <typename T>
__device__ __forceinline__ T strided_row(size_t base, uint32_t w, size_t stride,
                                         const uint32_t *__restrict__ cols,
                                         const T *__restrict__ elems, const T *__restrict__ x,
                                         int64_t xs, int64_t xinc) {
  T acc = strided_range<T>(T(0), base, 0, w, stride, cols, elems, x, xs, xinc);
  if (!finite_bits(acc)) acc = strided_row_skip<T>(base, w, stride, cols, elems, x, xs, xinc);
  return acc;
}

// ---------------------------------------------------------------------------
// ELL: thread per row, column-major slots (ell_matrix.hpp layout).
// ---------------------------------------------------------------------------
// W > 0: the width is a compile-time constant (one round, every load of the
// row issued up front); W == 0: runtime width.
template <int W, typename T>
__device__ __forceinline__ T ell_row(size_t r, uint32_t rows, uint32_t width,
                                     const uint32_t *__restrict__ coords,
                                     const T *__restrict__ elems, const T *__restrict__ x,
                                     int64_t xs, int64_t xinc) {
  if constexpr (W > 0) {
    T acc = strided_round<W>(T(0), r, 0, rows, coords, elems, x, xs, xinc);
    if (!finite_bits(acc)) acc = strided_row_skip<T>(r, W, rows, coords, elems, x, xs, xinc);
    return acc;
  } else {
    return strided_row<T>(r, width, rows, coords, elems, x, xs, xinc);
  }
}

template <int W, typename T, class E>
__global__ void __launch_bounds__(kSpmvThreads)
    ell_kernel(uint32_t rows, uint32_t width, const uint32_t *__restrict__ coords,
               const T *__restrict__ elems, const T *__restrict__ x, int64_t xs, int64_t xinc,
               E epi, T *partials, unsigned *counter) {
  pdl_trigger();
  pdl_wait();
  if (epi.skip()) return;
  __shared__ T smem[3 * (kSpmvThreads / 32) + 8];
  T dots[DotArr<E::NDOT>::n];
#pragma unroll
  for (int i = 0; i < DotArr<E::NDOT>::n; ++i) dots[i] = T(0);
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    const typename E::Pre pv = epi.pre((uint32_t)r);
    T acc = ell_row<W>(r, rows, width, coords, elems, x, xs, xinc);
    epi.row((uint32_t)r, acc, pv, dots);
  }
  if constexpr (E::NDOT > 0) {
    T sums[E::NDOT];
    if (grid_reduce<E::NDOT>(dots, partials, counter, smem, sums)) epi.finalize(sums);
  }
}

// ---------------------------------------------------------------------------
// DIA (internal format): thread per row; diagonal d contributes
// vals[d*rows + row] * x[row + off[d]] where that column exists, in ascending
// column order as a column-sorted CSR row.  ND > 0: the diagonal count is a
// compile-time constant and every value and x load of the row is issued
// before the first multiply (bounds tests only decide for boundary rows).
// ND == 0:
// any count up to kMaxDiag, one diagonal at a time.  x is contiguous (the
// inner solver's own vector).
// ---------------------------------------------------------------------------
template <int ND, typename T, class E>
__global__ void __launch_bounds__(kSpmvThreads)
    dia_kernel(uint32_t rows, uint32_t cols, DiaOffsets offs, const T *__restrict__ vals,
               const T *__restrict__ x, E epi, T *partials, unsigned *counter) {
  pdl_trigger();
  pdl_wait();
  if (epi.skip()) return;
  __shared__ T smem[3 * (kSpmvThreads / 32) + 8];
  T dots[DotArr<E::NDOT>::n];
#pragma unroll
  for (int i = 0; i < DotArr<E::NDOT>::n; ++i) dots[i] = T(0);
  // rows [lo, hi) have every diagonal inside the matrix
  const int64_t lo = -(int64_t)offs.off[0];
  const int64_t hi = (int64_t)cols - offs.off[offs.n - 1];
#pragma unroll 1
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    const typename E::Pre pv = epi.pre((uint32_t)r);
    // 32-bit indices: the DIA form is built only when rows, cols < 2^31 and
    // ndiag * rows < 2^32, so r + off cannot wrap into the valid range
    const uint32_t r32 = (uint32_t)r;
    T acc = T(0);
    if constexpr (ND > 0) {
      T v[ND], xv[ND];
      const bool inside = (int64_t)r >= lo && (int64_t)r < hi;
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        const uint32_t c = r32 + (uint32_t)offs.off[d];
        const bool in = inside || c < cols;
        v[d] = in ? __ldg(vals + (d * rows + r32)) : T(0);
        xv[d] = in ? __ldg(x + c) : T(0);
      }
#pragma unroll
      for (int d = 0; d < ND; ++d) acc += v[d] * xv[d];
    } else {
#pragma unroll 1
      for (int d = 0; d < offs.n; ++d) {
        const uint32_t c = r32 + (uint32_t)offs.off[d];
        if (c < cols) acc += __ldg(vals + (d * rows + r32)) * __ldg(x + c);
      }
    }
    epi.row((uint32_t)r, acc, pv, dots);
  }
  if constexpr (E::NDOT > 0) {
    T sums[E::NDOT];
    if (grid_reduce<E::NDOT>(dots, partials, counter, smem, sums)) epi.finalize(sums);
  }
}

// ---------------------------------------------------------------------------
// SELL-C-sigma: thread per stored row position; slice s, lane l; element j of
// the position at block_start[s] + j*C + l (sliced_ell_matrix.hpp layout).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T sell_row(size_t base, uint32_t w, uint32_t C,
                                      const uint32_t *__restrict__ cols,
                                      const T *__restrict__ elems, const T *__restrict__ x,
                                      int64_t xs, int64_t xinc) {
  return strided_row<T>(base, w, C, cols, elems, x, xs, xinc);
}

// WARP: C is a multiple of 32 and each warp takes 32 consecutive positions of
// one slice (no division per thread); the chunks listed in wide (all chunks of
// more than kSellWide slots, nwide of them) are taken by whole blocks instead.
// Otherwise thread per position.
template <bool WARP, typename T, class E>
__global__ void __launch_bounds__(kSpmvThreads)
    sell_kernel(uint32_t rows, uint32_t C, const uint32_t *__restrict__ cpb,
                const uint32_t *__restrict__ start, const uint32_t *__restrict__ cols,
                const T *__restrict__ elems, const uint32_t *__restrict__ perm,
                const uint32_t *__restrict__ wide, uint32_t nwide, const T *__restrict__ x,
                int64_t xs, int64_t xinc, E epi, T *partials, unsigned *counter) {
  pdl_trigger();
  pdl_wait();
  if (epi.skip()) return;
  __shared__ T smem[3 * (kSpmvThreads / 32) + 8];
  T dots[DotArr<E::NDOT>::n];
#pragma unroll
  for (int i = 0; i < DotArr<E::NDOT>::n; ++i) dots[i] = T(0);
  if constexpr (WARP) {
    constexpr uint32_t NW = kSpmvThreads / 32;
    __shared__ T part[NW][32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, per = C >> 5;
    const uint32_t nsub = (rows + 31) >> 5;  // 32-position chunks
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nsub;
         q += (gridDim.x * blockDim.x) >> 5) {
      const uint32_t s = q / per, l = (q - s * per) * 32 + lane;
      const uint32_t w = __ldg(cpb + s);
      if (nwide && w > kSellWide) continue;  // a block takes it below
      const uint32_t pos = q * 32 + lane;
      const uint32_t row = pos < rows ? (perm ? __ldg(perm + pos) : pos) : 0u;
      typename E::Pre pv{};
      if (pos < rows) pv = epi.pre(row);
      const T acc = sell_row(__ldg(start + s) + (size_t)l, w, C, cols, elems, x, xs, xinc);
      if (pos < rows) epi.row(row, acc, pv, dots);
    }
    for (uint32_t i = blockIdx.x; i < nwide; i += gridDim.x) {
      const uint32_t q = __ldg(wide + i), s = q / per, l = (q - s * per) * 32 + lane;
      const uint32_t w = __ldg(cpb + s);
      const size_t base = __ldg(start + s) + (size_t)l;
      const uint32_t j0 = (uint32_t)((uint64_t)w * warp / NW);
      const uint32_t j1 = (uint32_t)((uint64_t)w * (warp + 1) / NW);
      part[warp][lane] = strided_range<T>(T(0), base, j0, j1, C, cols, elems, x, xs, xinc);
      __syncthreads();
      if (warp == 0) {
        const uint32_t pos = q * 32 + lane;
        T acc = part[0][lane];
#pragma unroll
        for (uint32_t k = 1; k < NW; ++k) acc += part[k][lane];
        if (!finite_bits(acc)) acc = strided_row_skip<T>(base, w, C, cols, elems, x, xs, xinc);
        if (pos < rows) {
          const uint32_t row = perm ? __ldg(perm + pos) : pos;
          epi.row(row, acc, epi.pre(row), dots);
        }
      }
      __syncthreads();
    }
  } else {
    for (uint32_t pos = blockIdx.x * blockDim.x + threadIdx.x; pos < rows;
         pos += gridDim.x * blockDim.x) {
      const uint32_t s = pos / C, l = pos - s * C;
      const uint32_t row = perm ? __ldg(perm + pos) : pos;
      const typename E::Pre pv = epi.pre(row);
      const T acc = sell_row(__ldg(start + s) + (size_t)l, __ldg(cpb + s), C, cols, elems, x,
                             xs, xinc);
      epi.row(row, acc, pv, dots);
    }
  }
  if constexpr (E::NDOT > 0) {
    T sums[E::NDOT];
    if (grid_reduce<E::NDOT>(dots, partials, counter, smem, sums)) epi.finalize(sums);
  }
}

// ---------------------------------------------------------------------------
// HYB tail: COO entries (row-sorted) in chunks of 32*K per warp; lane l of the
// warp owns the K consecutive entries c0 + K*l ... of its chunk.  A lane sums
// its entries in order, row by row (one multiply and one add per entry); the
// rows that start and end inside a lane are complete and go to y at once.
// Only the lane's first and last row can continue into a neighbouring lane:
// one warp-segmented scan over the 32 lane partials (keyed by row) joins
// them.  The first and last row of every chunk can continue into the
// neighbouring chunk: they go to a carry array that hyb_tail_fixup adds in
// chunk order (deterministic, no atomics).  Per entry this costs about three
// FP64 instructions, against six for a scan over every entry.
// ---------------------------------------------------------------------------
constexpr int kTailK = 8;                       // consecutive entries per lane
constexpr int kTailChunk = 32 * kTailK;

// PAIRS: trow holds interleaved (row, col) pairs (coordinate_matrix's
// handle12 layout) and tcol is unused.
template <typename T, bool PAIRS = false>
__global__ void __launch_bounds__(kSpmvThreads)
    hyb_tail_kernel(uint64_t tnnz, const uint32_t *__restrict__ trow,
                    const uint32_t *__restrict__ tcol, const T *__restrict__ tval,
                    const T *__restrict__ x, int64_t xs, int64_t xinc, T alpha, T *y, int64_t ys,
                    int64_t yinc, uint32_t *carry_row, T *carry_val, const int *skip_flag) {
  if (skip_flag && *skip_flag) return;
  const uint32_t INV = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31;
  const size_t nchunks = (tnnz + kTailChunk - 1) / kTailChunk;
  const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t ch = warp; ch < nchunks; ch += nwarps) {
    const size_t c0 = ch * kTailChunk;
    const size_t c1 = c0 + kTailChunk < tnnz ? c0 + kTailChunk : tnnz;
    const uint32_t chunk_first = __ldg(trow + (PAIRS ? 2 * c0 : c0));
    const uint32_t chunk_last = __ldg(trow + (PAIRS ? 2 * (c1 - 1) : c1 - 1));
    const size_t e0 = c0 + (size_t)lane * kTailK;
    const uint32_t cnt = e0 < c1 ? (uint32_t)(c1 - e0 < (size_t)kTailK ? c1 - e0 : kTailK) : 0u;
    // every load of the lane's entries first, then its x gathers
    uint32_t r[kTailK], c[kTailK];
    T v[kTailK];
#pragma unroll
    for (int k = 0; k < kTailK; ++k) {
      const bool in = (uint32_t)k < cnt;
      if constexpr (PAIRS) {
        const uint2 rc = in ? __ldg(reinterpret_cast<const uint2 *>(trow) + e0 + k)
                            : make_uint2(INV, 0u);
        r[k] = rc.x;
        c[k] = rc.y;
      } else {
        r[k] = in ? __ldg(trow + e0 + k) : INV;
        c[k] = in ? __ldg(tcol + e0 + k) : 0u;
      }
      v[k] = in ? __ldg(tval + e0 + k) : T(0);
    }
    T p[kTailK];
#pragma unroll
    for (int k = 0; k < kTailK; ++k)
      p[k] = (uint32_t)k < cnt ? v[k] * __ldg(x + xs + (int64_t)c[k] * xinc) : T(0);
    // in-lane pass: first row's sum, complete interior rows, running last row
    const uint32_t first_row = r[0];
    uint32_t cur_row = r[0];
    T cur = p[0], first_sum = T(0);
    bool multi = false;
#pragma unroll
    for (int k = 1; k < kTailK; ++k) {
      if ((uint32_t)k < cnt) {
        if (r[k] == cur_row) {
          cur += p[k];
        } else {
          if (!multi) {
            first_sum = cur;
            multi = true;
          } else {  // starts and ends inside this lane: neither chunk end
            T *py = y + ys + (int64_t)cur_row * yinc;
            *py += alpha * cur;
          }
          cur_row = r[k];
          cur = p[k];
        }
      }
    }
    // segmented inclusive scan of the lanes' last-row partials; equal keys
    // are contiguous because the rows are sorted
    const uint32_t key = cur_row;
    T run = cur;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T q = __shfl_up_sync(0xffffffffu, run, o);
      const uint32_t qk = __shfl_up_sync(0xffffffffu, key, o);
      if ((int)lane >= o && qk == key) run += q;
    }
    const T prev_run = __shfl_up_sync(0xffffffffu, run, 1);
    const uint32_t prev_key = __shfl_up_sync(0xffffffffu, key, 1);
    const uint32_t next_first = __shfl_down_sync(0xffffffffu, first_row, 1);
    if (cnt > 0) {
      // a row that ends here: goes to the chunk's carry slots if it is the
      // chunk's first or last row, else straight to y
      auto emit = [&](uint32_t row, T total) {
        if (row == chunk_first) {
          carry_row[2 * ch] = row;
          carry_val[2 * ch] = total;
        } else if (row == chunk_last) {
          carry_row[2 * ch + 1] = row;
          carry_val[2 * ch + 1] = total;
        } else {
          T *py = y + ys + (int64_t)row * yinc;
          *py += alpha * total;
        }
      };
      if (multi) emit(first_row, (lane > 0 && prev_key == first_row) ? first_sum + prev_run : first_sum);
      if (lane == 31 || next_first != key) emit(key, run);
    }
    if (lane == 0 && chunk_first == chunk_last) carry_row[2 * ch + 1] = INV;
  }
}

// Adds the carries of the tail chunks: the chunk in which a row's tail starts
// owns the row and sums the continuation carries of the following chunks in
// order.  carry[2c] = first segment of chunk c, carry[2c+1] = last segment
// (0xffffffff when the chunk holds a single row).
template <typename T>
__global__ void hyb_tail_fixup(size_t nchunks, const uint32_t *__restrict__ carry_row,
                               const T *__restrict__ carry_val, T alpha, T *y, int64_t ys,
                               int64_t yinc, const int *skip_flag) {
  if (skip_flag && *skip_flag) return;
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < nchunks;
       c += (size_t)gridDim.x * blockDim.x) {
    for (int which = 0; which < 2; ++which) {
      uint32_t r = carry_row[2 * c + which];
      if (r == 0xffffffffu) continue;
      if (which == 0 && c > 0) {
        // continuation of a row owned by an earlier chunk?
        uint32_t pl = carry_row[2 * (c - 1) + 1];
        uint32_t pf = carry_row[2 * (c - 1)];
        uint32_t prev_last = (pl != 0xffffffffu) ? pl : pf;
        if (prev_last == r) continue;
      }
      T total = carry_val[2 * c + which];
      for (size_t d = c + 1; d < nchunks; ++d) {
        if (carry_row[2 * d] != r) break;
        total += carry_val[2 * d];
        if (carry_row[2 * d + 1] != 0xffffffffu) break;  // row ends inside chunk d
      }
      T *py = y + ys + (int64_t)r * yinc;
      *py += alpha * total;
    }
  }
}

// epilogue pass over an already computed product (HYB in the solvers)
template <typename T, class E>
__global__ void __launch_bounds__(kSpmvThreads)
    epilogue_pass_kernel(uint32_t rows, const T *__restrict__ y, E epi, T *partials,
                         unsigned *counter) {
  if (epi.skip()) return;
  __shared__ T smem[3 * (kSpmvThreads / 32) + 8];
  T dots[DotArr<E::NDOT>::n];
#pragma unroll
  for (int i = 0; i < DotArr<E::NDOT>::n; ++i) dots[i] = T(0);
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x)
    epi.row((uint32_t)r, y[r], epi.pre((uint32_t)r), dots);
  if constexpr (E::NDOT > 0) {
    T sums[E::NDOT];
    if (grid_reduce<E::NDOT>(dots, partials, counter, smem, sums)) epi.finalize(sums);
  }
}

// ---------------------------------------------------------------------------
// host-side dispatch
// ---------------------------------------------------------------------------
struct Reduction {
  void *partials = nullptr;  // >= NDOT (at most 4) * grid entries of T
  unsigned *counter = nullptr;
};

// grid of the SpMV kernels (also the number of partials per dot)
inline int spmv_grid(const Backend &be, const Matrix &m) {
  size_t work = m.format == VCLGB_SELL || m.format == VCLGB_ELL || m.format == kFormatDia
                    ? m.rows
                    : (m.rows + 3) / 4;
  if (m.format == VCLGB_CSR && m.nnz / 8 > work) work = m.nnz / 8;
  return waves_grid(be, kSpmvThreads, 8, work < 1 ? 1 : work);
}
constexpr int kMaxSpmvGrid = 152 * 8 * 2;

template <typename T, class E>
void ell_launch(Backend &be, int grid, const Matrix &m, const T *x, int64_t xs, int64_t xinc,
                const E &epi, T *partials, unsigned *counter) {
#define VCLGB_ELL(W)                                                                          \
  launch_kernel(be, ell_kernel<W, T, E>, one_wave<ell_kernel<W, T, E>>(be, grid, kSpmvThreads), \
                kSpmvThreads, 0, m.rows, m.ell_width, m.ell_coords.as<uint32_t>(),              \
                m.ell_elems.as<T>(), x, xs, xinc, epi, partials, counter)
  switch (m.ell_width) {
    case 1: VCLGB_ELL(1); break;
    case 2: VCLGB_ELL(2); break;
    case 3: VCLGB_ELL(3); break;
    case 4: VCLGB_ELL(4); break;
    case 5: VCLGB_ELL(5); break;
    case 6: VCLGB_ELL(6); break;
    case 7: VCLGB_ELL(7); break;
    case 8: VCLGB_ELL(8); break;
    default: VCLGB_ELL(0); break;
  }
#undef VCLGB_ELL
}

template <typename T, class E>
void spmv_launch(Backend &be, const Matrix &m0, const T *x, int64_t xs, int64_t xinc,
                 const E &epi, const Reduction &red, T *y_for_hyb = nullptr, int64_t ys = 0,
                 int64_t yinc = 1, T alpha = T(1), T beta = T(0), const int *skip_flag = nullptr,
                 void *hyb_scratch = nullptr) {
  const Matrix &m = spmv_form(m0);
  int grid = spmv_grid(be, m);
  T *partials = static_cast<T *>(red.partials);
  const int tp = timing_begin(be, 0);
  switch (m.format) {
    case VCLGB_CSR: {
      CsrView<T> A{m.row_ptr, m.col_idx, static_cast<const T *>(m.values), m.rows};
      const bool single = m.num_bins == 1 && m.bins[0].identity;
#define VCLGB_CSR_FIXED(L, R)                                                          \
  if constexpr (L == 1 && E::NDOT > 0 && std::is_same<T, double>::value)              \
    launch_kernel(be, csr_fixed_kernel<L, R, T, E, true>,                             \
                  one_wave<csr_fixed_kernel<L, R, T, E, true>>(be, grid, kSpmvThreads), \
                  kSpmvThreads, 0, A, x, xs, xinc, epi, partials, red.counter);       \
  else                                                                                \
    launch_kernel(be, csr_fixed_kernel<L, R, T, E>,                                   \
                  one_wave<csr_fixed_kernel<L, R, T, E>>(be, grid, kSpmvThreads),     \
                  kSpmvThreads, 0, A, x, xs, xinc, epi, partials, red.counter)
      const uint32_t lanes = single ? m.bins[0].lanes : 0u;
      if (lanes == 1) {
        switch (m.max_row_len) {
          case 3: VCLGB_CSR_FIXED(1, 3); break;
          case 4: VCLGB_CSR_FIXED(1, 4); break;
          case 5: VCLGB_CSR_FIXED(1, 5); break;
          case 6: VCLGB_CSR_FIXED(1, 6); break;
          case 7: VCLGB_CSR_FIXED(1, 7); break;
          default: VCLGB_CSR_FIXED(1, kMpl); break;
        }
      } else if (lanes == 2) {
        VCLGB_CSR_FIXED(2, kMpl);
      } else if (lanes == 4) {
        VCLGB_CSR_FIXED(4, kMpl);
      } else {
        const size_t nwin = (m.rows + kWinRows - 1) / kWinRows;
        const int wgrid = one_wave<csr_window_kernel<T, E>>(
            be, (int)(nwin < (size_t)grid ? (nwin ? nwin : 1) : grid), kSpmvThreads);
        launch_kernel(be, csr_window_kernel<T, E>, wgrid, kSpmvThreads, 0, A, x, xs, xinc, epi,
                      partials, red.counter);
      }
#undef VCLGB_CSR_FIXED
      break;
    }
    case VCLGB_ELL:
      ell_launch<T, E>(be, grid, m, x, xs, xinc, epi, partials, red.counter);
      break;
    case kFormatDia: {
      // the DIA form exists only as the refined solver's FP32 inner copy
      if constexpr (std::is_same<T, float>::value) {
        require(xs == 0 && xinc == 1, VCLGB_UNSUPPORTED, "DIA form takes a contiguous x");
        DiaOffsets o;
        o.n = (int)m.dia_ndiag;
        for (int d = 0; d < kMaxDiag; ++d) o.off[d] = m.dia_off[d];
#define VCLGB_DIA(ND)                                                                        \
  launch_kernel(be, dia_kernel<ND, T, E>, one_wave<dia_kernel<ND, T, E>>(be, grid, kSpmvThreads), \
                kSpmvThreads, 0, m.rows, m.cols, o, m.dia_vals.as<T>(), x, epi, partials,     \
                red.counter)
        switch (o.n) {
          case 3: VCLGB_DIA(3); break;
          case 5: VCLGB_DIA(5); break;
          case 7: VCLGB_DIA(7); break;
          case 9: VCLGB_DIA(9); break;
          default: VCLGB_DIA(0); break;
        }
#undef VCLGB_DIA
      } else {
        throw Error(VCLGB_UNSUPPORTED, "DIA form is an FP32 inner format");
      }
      break;
    }
    case VCLGB_SELL:
      if (m.C % 32 == 0)
        launch_kernel(be, sell_kernel<true, T, E>,
                      one_wave<sell_kernel<true, T, E>>(be, grid, kSpmvThreads), kSpmvThreads, 0,
            m.rows, m.C, m.sell_cpb.as<uint32_t>(), m.sell_start.as<uint32_t>(),
            m.sell_cols.as<uint32_t>(), m.sell_elems.as<T>(),
            m.sigma > 1 ? m.sell_perm.as<uint32_t>() : nullptr, m.sell_wide.as<uint32_t>(),
            m.sell_nwide, x, xs, xinc, epi, partials, red.counter);
      else
        launch_kernel(be, sell_kernel<false, T, E>,
                      one_wave<sell_kernel<false, T, E>>(be, grid, kSpmvThreads), kSpmvThreads, 0,
            m.rows, m.C, m.sell_cpb.as<uint32_t>(), m.sell_start.as<uint32_t>(),
            m.sell_cols.as<uint32_t>(), m.sell_elems.as<T>(),
            m.sigma > 1 ? m.sell_perm.as<uint32_t>() : nullptr, nullptr, 0u, x, xs, xinc, epi,
            partials, red.counter);
      break;
    case VCLGB_HYB:
    case VCLGB_COO: {
      // y = alpha*ELL*x + beta*y, then y += alpha*tail*x, then the epilogue
      // pass; COO is the case of an empty ELL part (width 0: the first pass
      // only scales y) and a tail of all entries
      with_axpby_mode(alpha, beta, [&](auto mode) {
        constexpr int MODE = decltype(mode)::value;
        auto part = [&](auto sp) {
          sp.alpha = alpha; sp.beta = beta; sp.y = y_for_hyb; sp.ys = ys; sp.yinc = yinc;
          sp.flag = skip_flag;
          ell_launch<T, decltype(sp)>(be, grid, m, x, xs, xinc, sp, partials, red.counter);
        };
        if (ys == 0 && yinc == 1) part(EpiAxpbySkip<T, MODE, true>{});
        else part(EpiAxpbySkip<T, MODE, false>{});
      });
      if (m.tail_nnz > 0) {
        size_t nchunks = (m.tail_nnz + kTailChunk - 1) / kTailChunk;
        uint32_t *carry_row = static_cast<uint32_t *>(hyb_scratch);
        T *carry_val = reinterpret_cast<T *>(static_cast<char *>(hyb_scratch) +
                                             ((2 * nchunks * sizeof(uint32_t) + 15) / 16) * 16);
        const int g0 = waves_grid(be, kSpmvThreads, 8, nchunks * 32);
        if (m.format == VCLGB_COO)
          hyb_tail_kernel<T, true>
              <<<one_wave<hyb_tail_kernel<T, true>>(be, g0, kSpmvThreads), kSpmvThreads, 0,
                 be.stream>>>(m.tail_nnz, m.coo_coords.as<uint32_t>(), nullptr,
                              m.coo_elems.as<T>(), x, xs, xinc, alpha, y_for_hyb, ys, yinc,
                              carry_row, carry_val, skip_flag);
        else
          hyb_tail_kernel<T, false>
              <<<one_wave<hyb_tail_kernel<T, false>>(be, g0, kSpmvThreads), kSpmvThreads, 0,
                 be.stream>>>(m.tail_nnz, m.tail_row.as<uint32_t>(), m.tail_ci.as<uint32_t>(),
                              m.tail_v.as<T>(), x, xs, xinc, alpha, y_for_hyb, ys, yinc,
                              carry_row, carry_val, skip_flag);
        int g2 = (int)((nchunks + 255) / 256);
        hyb_tail_fixup<T><<<g2, 256, 0, be.stream>>>(nchunks, carry_row, carry_val, alpha,
                                                      y_for_hyb, ys, yinc, skip_flag);
        be.launches += 2;
      }
      if constexpr (E::NDOT > 0) {
        epilogue_pass_kernel<T, E><<<one_wave<epilogue_pass_kernel<T, E>>(be, grid, kSpmvThreads),
                                     kSpmvThreads, 0, be.stream>>>(
            m.rows, y_for_hyb, epi, partials, red.counter);
        be.launches++;
      }
      break;
    }
  }
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  timing_end(be, tp);
}

// scratch bytes the HYB tail needs (carry arrays), for the form a product runs on
inline size_t hyb_scratch_bytes(const Matrix &m0) {
  const Matrix &m = spmv_form(m0);
  if ((m.format != VCLGB_HYB && m.format != VCLGB_COO) || m.tail_nnz == 0) return 0;
  size_t nchunks = (m.tail_nnz + kTailChunk - 1) / kTailChunk;
  return ((2 * nchunks * sizeof(uint32_t) + 15) / 16) * 16 + 2 * nchunks * 8 + 16;
}

}  // namespace vclgb
