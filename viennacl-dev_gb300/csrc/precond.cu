// precond.cu -- Jacobi and ILU0 preconditioners.
//
// Jacobi: diag(A) by a device kernel (row_info SPARSE_ROW_DIAGONAL,
// linalg/cuda/sparse_matrix_operations.hpp:53-119); apply z = r / diag is fused
// into the solvers' update kernels.
//
// ILU0 (linalg/detail/ilu/ilu0.hpp): the elimination levels of L and U and
// the per-level substitution lists follow level_scheduling_setup_impl
// (detail/ilu/common.hpp:50-187) and are built from the pattern on the host,
// as the reference does; the numeric factorisation then runs on the device,
// level by level (rows of one level are independent; a run of small levels is
// one single-block launch with a barrier between levels), with the same
// per-row IKJ operation order and no fused multiply-add, so the factors are
// bit-identical to the reference's sequential host loop (ilu0.hpp:77-140).
// The apply substitutes level by level (linalg/cuda/misc_operations.hpp:41-83
// semantics): a run of small levels is one block (level_run_kernel), a large
// level one grid-wide launch (level_substitute_kernel).
#include <algorithm>
#include <exception>
#include <map>
#include <thread>

#include <cooperative_groups.h>

#include "formats.hpp"
#include "vecpass.cuh"

namespace cg = cooperative_groups;

namespace vclgb {

template <typename T>
__global__ void diag_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                            const uint32_t *__restrict__ ci, const T *__restrict__ v, T *d,
                            unsigned *zero_found) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    T val = 0;
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k)
      if (ci[k] == r) { val = v[k]; break; }
    d[r] = val;
    if (zero_found && val == T(0)) atomicOr(zero_found, 1u);
  }
}

void extract_diag(Backend &be, const Matrix &A, DevBuf &out, bool check_zero) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "diagonal extraction needs CSR");
  out.alloc(std::max<size_t>(A.rows, 1) * A.vsize(), be.stream);
  DevBuf flag(sizeof(unsigned), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(unsigned), be.stream));
  int g = waves_grid(be, 256, 8, A.rows);
  if (A.prec == VCLGB_FLOAT64)
    diag_kernel<double><<<g, 256, 0, be.stream>>>(A.rows, A.row_ptr, A.col_idx,
                                                  static_cast<const double *>(A.values),
                                                  out.as<double>(), flag.as<unsigned>());
  else
    diag_kernel<float><<<g, 256, 0, be.stream>>>(A.rows, A.row_ptr, A.col_idx,
                                                 static_cast<const float *>(A.values),
                                                 out.as<float>(), flag.as<unsigned>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  if (check_zero) {
    unsigned h = 0;
    VCLGB_CUDA(cudaMemcpyAsync(&h, flag.ptr, sizeof(h), cudaMemcpyDeviceToHost, be.stream));
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    if (h) throw Error(VCLGB_ZERO_ON_DIAGONAL, "zero on diagonal");
  }
}

template <typename T>
__global__ void recip_kernel(size_t n, const T *__restrict__ d, T *inv) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    inv[i] = T(1) / d[i];
}

// 1 / diag of a diagonal preconditioner, formed once: the fused solver
// kernels multiply by it (an FP64 division is a sequence of FP64-pipe
// instructions on GB300; dividing every row in every iteration made the
// Jacobi-PCG update kernel FP64-bound at a quarter of HBM speed).  The
// products differ from the reference's element_div by at most an ulp;
// vclgbPrecondApply keeps the division.
static void make_inv_diag(Backend &be, Precond &P) {
  P.inv_diag.alloc(std::max<size_t>(P.rows, 1) * (P.prec == VCLGB_FLOAT64 ? 8 : 4), be.stream);
  if (!P.rows) return;
  const int g = waves_grid(be, 256, 8, P.rows);
  if (P.prec == VCLGB_FLOAT64)
    recip_kernel<double><<<g, 256, 0, be.stream>>>(P.rows, P.diag.as<double>(), P.inv_diag.as<double>());
  else
    recip_kernel<float><<<g, 256, 0, be.stream>>>(P.rows, P.diag.as<float>(), P.inv_diag.as<float>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
}

std::unique_ptr<Precond> jacobi_create(Backend &be, const Matrix &A) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "jacobi_precond is built from CSR");
  auto P = std::make_unique<Precond>();
  P->kind = 1;
  P->prec = A.prec;
  P->rows = A.rows;
  extract_diag(be, A, P->diag, true);
  make_inv_diag(be, *P);
  return P;
}

// ---------------------------------------------------------------------------
// row_scaling (linalg/row_scaling.hpp:150-191): a diagonal preconditioner
// whose entries are row norms of A, from row_info SPARSE_ROW_NORM_INF / _1 / _2
// (linalg/host_based/sparse_matrix_operations.hpp:52-98): rows summed in
// storage order with separate multiply and add (no fused multiply-add), so
// the norms equal the reference's bit for bit.  The apply is Jacobi's
// element_div, fused into the solvers in the same way.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <>
__device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }
template <typename T>
__device__ __forceinline__ T sqr_rn(T a);
template <>
__device__ __forceinline__ double sqr_rn<double>(double a) { return __dmul_rn(a, a); }
template <>
__device__ __forceinline__ float sqr_rn<float>(float a) { return __fmul_rn(a, a); }

template <typename T>
__global__ void row_norm_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                const T *__restrict__ v, uint32_t norm, T *d) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    T value = 0;
    const uint32_t e = rp[r + 1];
    if (norm == 0) {
      for (uint32_t k = rp[r]; k < e; ++k) {
        const T a = fabs(v[k]);
        value = value < a ? a : value;  // std::max(value, |a|)
      }
    } else if (norm == 1) {
      for (uint32_t k = rp[r]; k < e; ++k) value = add_rn(value, T(fabs(v[k])));
    } else {
      for (uint32_t k = rp[r]; k < e; ++k) value = add_rn(value, sqr_rn(v[k]));
      value = sqrt(value);
    }
    d[r] = value;
  }
}

std::unique_ptr<Precond> row_scaling_create(Backend &be, const Matrix &A, uint32_t norm) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "row_scaling is built from CSR");
  require(norm <= 2, VCLGB_INVALID_ARGUMENT,
          "unknown norm for row_scaling (0 = max, 1 = sum, 2 = Euclidean)");
  auto P = std::make_unique<Precond>();
  P->kind = 1;  // a diagonal, applied like Jacobi's
  P->prec = A.prec;
  P->rows = A.rows;
  P->diag.alloc(std::max<size_t>(A.rows, 1) * A.vsize(), be.stream);
  if (A.rows) {
    int g = waves_grid(be, 256, 8, A.rows);
    if (A.prec == VCLGB_FLOAT64)
      row_norm_kernel<double><<<g, 256, 0, be.stream>>>(
          A.rows, A.row_ptr, static_cast<const double *>(A.values), norm, P->diag.as<double>());
    else
      row_norm_kernel<float><<<g, 256, 0, be.stream>>>(
          A.rows, A.row_ptr, static_cast<const float *>(A.values), norm, P->diag.as<float>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  }
  make_inv_diag(be, *P);
  return P;
}

// ---------------------------------------------------------------------------
// ILU0
// ---------------------------------------------------------------------------
// numeric factorisation of the rows of one level (thread per row)
template <typename T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <typename T>
__device__ __forceinline__ T sub_rn(T a, T b);
template <>
__device__ __forceinline__ double sub_rn<double>(double a, double b) { return __dsub_rn(a, b); }
template <>
__device__ __forceinline__ float sub_rn<float>(float a, float b) { return __fsub_rn(a, b); }

// the factorisation of one row, in the reference's IKJ order (ilu0.hpp:77-140)
template <typename T>
__device__ __forceinline__ void ilu0_row_generic(uint32_t i, const uint32_t *__restrict__ rp,
                                                 const uint32_t *__restrict__ ci, T *lu) {
  const uint32_t ib = rp[i], ie = rp[i + 1];
  for (uint32_t bk = ib; bk < ie; ++bk) {
    const uint32_t k = ci[bk];
    if (k >= i) continue;
    const uint32_t kb = rp[k], ke = rp[k + 1];
    T a_kk = 0;
    for (uint32_t q = kb; q < ke; ++q)
      if (ci[q] == k) { a_kk = lu[q]; break; }
    const T a_ik = lu[bk] / a_kk;
    lu[bk] = a_ik;
    for (uint32_t bj = ib; bj < ie; ++bj) {
      const uint32_t j = ci[bj];
      if (j <= k) continue;
      T a_kj = 0;
      for (uint32_t q = kb; q < ke; ++q)
        if (ci[q] == j) { a_kj = lu[q]; break; }
      lu[bj] = sub_rn(lu[bj], mul_rn(a_ik, a_kj));
    }
  }
}

// The same row with row i and the first kRowCache entries of each row k in
// registers: each row is read in one round of independent loads instead of a
// chain of dependent ones, row i is written back once at the end (no other
// thread reads it while its level runs), and a value of row k is the first
// match in storage order -- cached entries first, the rest of a longer row k
// from memory -- so every operation and its operands are the generic path's.
constexpr int kRowCache = 8;

template <typename T>
__device__ __forceinline__ T ilu0_lookup(uint32_t j, const uint32_t (&kc)[kRowCache],
                                         const T (&kv)[kRowCache], uint32_t kb, uint32_t ke,
                                         const uint32_t *__restrict__ ci, const T *lu) {
  bool found = false;
  T v = T(0);
#pragma unroll
  for (int q = 0; q < kRowCache; ++q)
    if (!found && kc[q] == j) {
      v = kv[q];
      found = true;
    }
  if (!found)
    for (uint32_t q = kb + kRowCache; q < ke; ++q)
      if (ci[q] == j) { v = lu[q]; break; }
  return v;
}

template <typename T>
__device__ __forceinline__ void ilu0_row(uint32_t i, const uint32_t *__restrict__ rp,
                                         const uint32_t *__restrict__ ci, T *lu) {
  const uint32_t ib = rp[i], ie = rp[i + 1], len = ie - ib;
  if (len > (uint32_t)kRowCache) {
    ilu0_row_generic<T>(i, rp, ci, lu);
    return;
  }
  uint32_t c[kRowCache];
  T a[kRowCache];
#pragma unroll
  for (int t = 0; t < kRowCache; ++t) {
    const bool on = (uint32_t)t < len;
    c[t] = on ? ci[ib + t] : 0xffffffffu;
    a[t] = on ? lu[ib + t] : T(0);
  }
#pragma unroll
  for (int tk = 0; tk < kRowCache; ++tk) {
    const uint32_t k = c[tk];
    if ((uint32_t)tk >= len || k >= i) continue;
    const uint32_t kb = rp[k], ke = rp[k + 1];
    uint32_t kc[kRowCache];
    T kv[kRowCache];
#pragma unroll
    for (int q = 0; q < kRowCache; ++q) {
      const bool on = kb + q < ke;
      kc[q] = on ? ci[kb + q] : 0xffffffffu;
      kv[q] = on ? lu[kb + q] : T(0);
    }
    const T a_kk = ilu0_lookup<T>(k, kc, kv, kb, ke, ci, lu);
    const T a_ik = a[tk] / a_kk;
    a[tk] = a_ik;
#pragma unroll
    for (int tj = 0; tj < kRowCache; ++tj) {
      const uint32_t j = c[tj];
      if ((uint32_t)tj >= len || j <= k) continue;
      a[tj] = sub_rn(a[tj], mul_rn(a_ik, ilu0_lookup<T>(j, kc, kv, kb, ke, ci, lu)));
    }
  }
#pragma unroll
  for (int t = 0; t < kRowCache; ++t)
    if ((uint32_t)t < len) lu[ib + t] = a[t];
}

template <typename T>
__global__ void ilu0_level_kernel(uint32_t count, const uint32_t *__restrict__ rows_of_level,
                                  const uint32_t *__restrict__ rp,
                                  const uint32_t *__restrict__ ci, T *lu) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += (size_t)gridDim.x * blockDim.x)
    ilu0_row<T>(rows_of_level[t], rp, ci, lu);
}

// consecutive levels [e0, e1) of at most kFactorRun rows each in one block,
// a barrier between levels: a row reads only rows of earlier levels, which
// this block finished before a barrier.  Level e's rows are
// order[off[e] .. off[e + 1]).  512 threads leave the cached row update room
// for its registers (at 1024 threads the FP64 version spills).
constexpr uint32_t kFactorRun = 512;

template <typename T>
__global__ void __launch_bounds__(kFactorRun, 1)
    ilu0_run_kernel(uint32_t e0, uint32_t e1, const uint32_t *__restrict__ off,
                    const uint32_t *__restrict__ order, const uint32_t *__restrict__ rp,
                    const uint32_t *__restrict__ ci, T *lu) {
  for (uint32_t e = e0; e < e1; ++e) {
    const uint32_t t = __ldg(off + e) + threadIdx.x;
    if (t < __ldg(off + e + 1)) ilu0_row<T>(__ldg(order + t), rp, ci, lu);
    __syncthreads();
  }
}

// gather of the level-set values from the factors (U scaled by its diagonal),
// one thread per level row
template <typename T>
__global__ void level_vals_kernel(size_t level_rows, const uint32_t *__restrict__ row_index,
                                  const uint32_t *__restrict__ row_ptr,
                                  const uint32_t *__restrict__ src, const T *__restrict__ lu,
                                  const T *__restrict__ udiag, T *vals) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < level_rows;
       t += (size_t)gridDim.x * blockDim.x) {
    const T d = udiag ? udiag[row_index[t]] : T(1);
    for (uint32_t k = row_ptr[t]; k < row_ptr[t + 1]; ++k) {
      T v = lu[src[k]];
      if (udiag) v = v / d;
      vals[k] = v;
    }
  }
}

// one level: vec[row] -= sum vals * vec[cols] (misc_operations.hpp substitute)
template <typename T>
__global__ void level_substitute_kernel(uint32_t r0, uint32_t r1,
                                        const uint32_t *__restrict__ row_index,
                                        const uint32_t *__restrict__ row_ptr,
                                        const uint32_t *__restrict__ cols,
                                        const T *__restrict__ vals, T *vec, const int *skip) {
  if (skip && *skip) return;
  for (size_t t = r0 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < r1;
       t += (size_t)gridDim.x * blockDim.x) {
    const uint32_t row = row_index[t];
    T s = vec[row];
    for (uint32_t j = row_ptr[t]; j < row_ptr[t + 1]; ++j) s -= vec[cols[j]] * vals[j];
    vec[row] = s;
  }
}

template <typename T>
__global__ void div_kernel(size_t n, T *vec, const T *__restrict__ d, const int *skip) {
  if (skip && *skip) return;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    vec[i] = vec[i] / d[i];
}

// level structure of one triangle (host, from the pattern)
struct LevelPlan {
  std::vector<uint32_t> level_ptr, row_index, row_ptr, cols, src;
  // ring codes of the runs of small levels (plan_codes), run_width 0: none
  std::vector<int32_t> ecode, xcode;
  uint32_t run_width = 0;
};

static LevelPlan plan_levels(uint32_t n, const std::vector<uint32_t> &rp,
                             const std::vector<uint32_t> &ci, bool upper,
                             std::vector<uint32_t> *row_level_out) {
  std::vector<uint32_t> lev(n, 0);
  uint32_t maxlev = 0;
  for (uint32_t r2 = 0; r2 < n; ++r2) {
    uint32_t row = upper ? n - 1 - r2 : r2, e = 0;
    for (uint32_t k = rp[row]; k < rp[row + 1]; ++k) {
      uint32_t c = ci[k];
      if ((!upper && c < row) || (upper && c > row)) e = std::max(e, lev[c]);
    }
    lev[row] = e + 1;
    maxlev = std::max(maxlev, e + 1);
  }
  // bucket entries by the level of their column; rows ascending inside a level
  std::vector<uint64_t> cnt_rows(maxlev + 2, 0), cnt_nnz(maxlev + 2, 0);
  std::vector<uint32_t> seen(maxlev + 2, 0);
  for (uint32_t row = 0; row < n; ++row)
    for (uint32_t k = rp[row]; k < rp[row + 1]; ++k) {
      uint32_t c = ci[k];
      if ((!upper && c < row) || (upper && c > row)) {
        uint32_t e = lev[c];
        cnt_nnz[e] += 1;
        if (seen[e] != row + 1) { seen[e] = row + 1; cnt_rows[e] += 1; }
      }
    }
  LevelPlan p;
  // per-level cursors
  std::vector<uint64_t> row_off(maxlev + 2, 0), nnz_off(maxlev + 2, 0);
  uint64_t ro = 0, no = 0;
  p.level_ptr.push_back(0);
  for (uint32_t e = 1; e <= maxlev; ++e) {
    if (cnt_rows[e] == 0) continue;
    row_off[e] = ro;
    nnz_off[e] = no;
    ro += cnt_rows[e];
    no += cnt_nnz[e];
    p.level_ptr.push_back((uint32_t)ro);
  }
  p.row_index.assign(ro, 0);
  p.row_ptr.assign(ro + 1, 0);
  p.cols.assign(no, 0);
  p.src.assign(no, 0);
  // rows are visited in ascending order, so each level's list stays sorted,
  // and a row's entries of one level are appended together: its row pointer
  // is the level's entry cursor when the row first reaches the level
  std::vector<uint64_t> rcur(row_off), ncur(nnz_off);
  std::fill(seen.begin(), seen.end(), 0);
  for (uint32_t row = 0; row < n; ++row) {
    for (uint32_t k = rp[row]; k < rp[row + 1]; ++k) {
      const uint32_t c = ci[k];
      if (!((!upper && c < row) || (upper && c > row))) continue;
      const uint32_t e = lev[c];
      if (seen[e] != row + 1) {
        seen[e] = row + 1;
        p.row_index[rcur[e]] = row;
        p.row_ptr[rcur[e]] = (uint32_t)ncur[e];
        rcur[e] += 1;
      }
      p.cols[ncur[e]] = c;
      p.src[ncur[e]] = k;
      ncur[e] += 1;
    }
  }
  p.row_ptr[ro] = (uint32_t)no;
  if (row_level_out) *row_level_out = std::move(lev);
  return p;
}

// Runs of small levels: consecutive levels of at most run_width rows each are
// substituted by one launch -- one block (level_run_kernel, levels of at most
// kRunLevel rows) or one thread-block cluster (level_cluster_kernel, up to
// kCodeWidth rows) -- with a barrier between levels; the values written in the
// last kRing levels of a run stay in shared memory.  A read's ring code names
// level e's position p as (e mod kRing) * kCodeWidth + p; the block keeps its
// ring as kRing x kRunLevel slots, a cluster spreads it over its CTAs.
constexpr uint32_t kRunLevel = 1024;
constexpr uint32_t kCodeWidth = 16384;  // the widest cluster: 16 CTAs x 1024 threads
constexpr uint32_t kCodeShift = 14;
static_assert((1u << kCodeShift) == kCodeWidth, "code width");
constexpr uint32_t kRing = 16;
constexpr uint32_t kRingSlots = kRing * kRunLevel;
static_assert((kRingSlots & (kRingSlots - 1)) == 0, "ring slots index by mask");

// first level at or after L with more than `width` rows (L itself if L has)
static uint32_t run_end(const std::vector<uint32_t> &level_ptr, uint32_t L, uint32_t width) {
  const uint32_t levels = (uint32_t)level_ptr.size() - 1;
  if (width == 0) return L;
  while (L < levels && level_ptr[L + 1] - level_ptr[L] <= width) ++L;
  return L;
}

// the widest level of levels [L, L1)
static uint32_t widest_level(const std::vector<uint32_t> &level_ptr, uint32_t L, uint32_t L1) {
  uint32_t w = 0;
  for (uint32_t e = L; e < L1; ++e) w = std::max(w, level_ptr[e + 1] - level_ptr[e]);
  return w;
}

// Where each read of a run finds its value: a code < 0 is ring slot ~code
// (the row was last written at most kRing - 1 levels earlier in the same run),
// a code >= 0 is the row to read from the vector in global memory (written
// before the run, by a large level, or at least kRing levels earlier -- so
// the value is final there, a barrier at least one level back).  ecode per
// entry (the column's value), xcode per level row (the row's own value).
static void plan_ring_codes(const std::vector<uint32_t> &level_ptr,
                            const std::vector<uint32_t> &row_index,
                            const std::vector<uint32_t> &row_ptr, const std::vector<uint32_t> &cols,
                            uint32_t n, uint32_t run_width, std::vector<int32_t> &ecode,
                            std::vector<int32_t> &xcode) {
  const uint32_t levels = (uint32_t)level_ptr.size() - 1;
  ecode.resize(cols.size());
  xcode.resize(row_index.size());
  // per row: level, position and run of its last write (run 0: none), in one
  // record so a lookup touches one cache line
  struct Written {
    uint32_t lev, pos, run;
  };
  std::vector<Written> w(n, Written{0, 0, 0});
  uint32_t run = 0;
  for (uint32_t L = 0; L < levels;) {
    uint32_t L1 = run_end(level_ptr, L, run_width);
    const bool small = L1 > L;
    if (!small) L1 = L + 1;
    ++run;
    for (uint32_t e = L; e < L1; ++e) {
      auto code = [&](uint32_t r) -> int32_t {
        const Written &x = w[r];
        if (small && x.run == run && e - x.lev < kRing)
          return ~(int32_t)((x.lev % kRing) * kCodeWidth + x.pos);
        return (int32_t)r;
      };
      for (uint32_t t = level_ptr[e]; t < level_ptr[e + 1]; ++t) {
        xcode[t] = code(row_index[t]);
        for (uint32_t j = row_ptr[t]; j < row_ptr[t + 1]; ++j) ecode[j] = code(cols[j]);
      }
      for (uint32_t t = level_ptr[e]; t < level_ptr[e + 1]; ++t) {
        w[row_index[t]] = Written{e, t - level_ptr[e], small ? run : 0};
      }
    }
    L = L1;
  }
}

// the ring codes of a plan's runs of levels of at most run_width rows (host
// only, so that it can run beside the device work of another triangle)
static void plan_codes(LevelPlan &pl, uint32_t n, uint32_t run_width) {
  pl.run_width = n >= 0x80000000u ? 0 : run_width;  // codes hold a row index in an int32
  if (pl.run_width)
    plan_ring_codes(pl.level_ptr, pl.row_index, pl.row_ptr, pl.cols, n, pl.run_width, pl.ecode,
                    pl.xcode);
}

// level_run_kernel: a run of consecutive small levels, one block; a level is
// one pass of the block and a __syncthreads() replaces the kernel launch
// between levels.  On a 2D grid every level is an anti-diagonal of at most a
// few hundred rows, so a whole triangle is one launch instead of 2*sqrt(n).
//
// A level holds, for each row, the entries whose columns lie in it (a row is
// updated at every level its columns reach).  The values the level reads come
// from the ring when they were written in the last kRing levels of the run
// (on a stencil: all of them, one level back), else from global memory, where
// they are final since at least one barrier -- which is why a global read of
// the row's own value can be issued early.  The pattern is read-only: with NT
// threads, a level's entries (first kRunPre codes and values, the row's own
// global value) are fetched DE levels ahead and its row information 2 DE
// levels ahead.  DE = 1 fits 1024 threads in 64 registers; runs whose levels
// hold at most 512 rows take 512 threads and DE = 4, which gives every
// pattern load four levels to arrive (an early global read of the row's own
// value is safe while DE < kRing).  Each row subtracts the same entries in the
// same order as level_substitute_kernel, so the results do not depend on
// which kernel ran.
constexpr int kRunPre = 3;
constexpr uint32_t kNoRow = 0xffffffffu;

struct RunRow {
  uint32_t row, jb, je;  // row == kNoRow when the thread has no row in the level
  int32_t xc;            // where the row's own value is (plan_ring_codes)
};

template <typename T>
struct RunEntries {
  RunRow r;
  int32_t c[kRunPre];
  T v[kRunPre];
  T xg;  // the row's value, prefetched when it lies in global memory
};

__device__ __forceinline__ RunRow run_fetch_row(uint32_t lev, uint32_t lev1,
                                                const uint32_t *__restrict__ level_ptr,
                                                const uint32_t *__restrict__ row_index,
                                                const int32_t *__restrict__ xcode,
                                                const uint32_t *__restrict__ row_ptr,
                                                uint32_t pos) {
  RunRow r{kNoRow, 0, 0, 0};
  if (lev < lev1) {
    const uint32_t t = __ldg(level_ptr + lev) + pos;
    if (t < __ldg(level_ptr + lev + 1)) {
      r.row = __ldg(row_index + t);
      r.jb = __ldg(row_ptr + t);
      r.je = __ldg(row_ptr + t + 1);
      r.xc = __ldg(xcode + t);
    }
  }
  return r;
}

template <typename T, bool L2 = false>
__device__ __forceinline__ RunEntries<T> run_fetch_entries(RunRow r,
                                                           const int32_t *__restrict__ ecode,
                                                           const T *__restrict__ vals,
                                                           const T *vec) {
  RunEntries<T> e;
  e.r = r;
#pragma unroll
  for (int k = 0; k < kRunPre; ++k) {
    const bool on = r.jb + k < r.je;
    e.c[k] = on ? __ldg(ecode + r.jb + k) : 0;
    e.v[k] = on ? __ldg(vals + r.jb + k) : T(0);
  }
  e.xg = (r.row != kNoRow && r.xc >= 0) ? (L2 ? __ldcg(vec + r.xc) : vec[r.xc]) : T(0);
  return e;
}

// ring slot of code g in a block's ring (positions below kRunLevel)
__device__ __forceinline__ uint32_t block_slot(uint32_t g) {
  return ((g >> kCodeShift) & (kRing - 1)) * kRunLevel + (g & (kRunLevel - 1));
}

template <typename T>
__device__ __forceinline__ T run_read(int32_t code, const T *ring, const T *vec) {
  return code < 0 ? ring[block_slot((uint32_t)~code)] : vec[code];
}

// one level of a run: consume the entries of level lev from `ent`, refill it
// with level lev + DE (its row information is in `row`) and refill `row` with
// level lev + 2 DE.  The caller unrolls its level loop by DE, so that every
// stage keeps its registers (stage lev mod DE) and nothing is moved between
// levels.
template <typename T, int DE>
__device__ __forceinline__ void run_level(uint32_t lev, uint32_t lev1, RunEntries<T> &ent,
                                          RunRow &row, const uint32_t *__restrict__ level_ptr,
                                          const uint32_t *__restrict__ row_index,
                                          const int32_t *__restrict__ xcode,
                                          const uint32_t *__restrict__ row_ptr,
                                          const int32_t *__restrict__ ecode,
                                          const T *__restrict__ vals, T *vec, T *ring) {
  const RunRow r = ent.r;
  T x = T(0), y[kRunPre];
  if (r.row != kNoRow) x = r.xc >= 0 ? ent.xg : ring[block_slot((uint32_t)~r.xc)];
#pragma unroll
  for (int k = 0; k < kRunPre; ++k) y[k] = r.jb + k < r.je ? run_read(ent.c[k], ring, vec) : T(0);
  T s = x;
  if (r.row != kNoRow) {
#pragma unroll
    for (int k = 0; k < kRunPre; ++k)
      if (r.jb + k < r.je) s -= y[k] * ent.v[k];
    for (uint32_t j = r.jb + kRunPre; j < r.je; ++j)
      s -= run_read(__ldg(ecode + j), ring, vec) * __ldg(vals + j);
    ring[(lev & (kRing - 1)) * kRunLevel + threadIdx.x] = s;
  }
  ent = run_fetch_entries<T>(row, ecode, vals, vec);
  row = run_fetch_row(lev + 2 * DE, lev1, level_ptr, row_index, xcode, row_ptr, threadIdx.x);
  __syncthreads();
  // the global copy is read only kRing levels later (or after the kernel),
  // so it is stored after the barrier, off the level's critical path
  if (r.row != kNoRow) vec[r.row] = s;
}

template <typename T, uint32_t NT, int DE>
__global__ void __launch_bounds__(NT)
    level_run_kernel(uint32_t lev0, uint32_t lev1, const uint32_t *__restrict__ level_ptr,
                     const uint32_t *__restrict__ row_index, const int32_t *__restrict__ xcode,
                     const uint32_t *__restrict__ row_ptr, const int32_t *__restrict__ ecode,
                     const T *__restrict__ vals, T *vec, const int *skip) {
  static_assert(DE >= 1 && DE < (int)kRing && NT <= kRunLevel, "pipeline depth and width");
  extern __shared__ __align__(16) unsigned char ring_bytes[];
  T *ring = reinterpret_cast<T *>(ring_bytes);
  if (skip && *skip) return;
  RunEntries<T> ents[DE];  // stage k: level lev0 + k, then every DE levels on
  RunRow rows[DE];         // stage k: DE levels ahead of ents[k]
#pragma unroll
  for (int k = 0; k < DE; ++k)
    ents[k] = run_fetch_entries<T>(
        run_fetch_row(lev0 + k, lev1, level_ptr, row_index, xcode, row_ptr, threadIdx.x), ecode,
        vals, vec);
#pragma unroll
  for (int k = 0; k < DE; ++k)
    rows[k] = run_fetch_row(lev0 + DE + k, lev1, level_ptr, row_index, xcode, row_ptr,
                            threadIdx.x);
  for (uint32_t lev = lev0; lev < lev1; lev += DE) {
#pragma unroll
    for (int k = 0; k < DE; ++k) {
      if (lev + k >= lev1) break;  // uniform over the block
      run_level<T, DE>(lev + k, lev1, ents[k], rows[k], level_ptr, row_index, xcode, row_ptr,
                       ecode, vals, vec, ring);
    }
  }
}

// Cluster runs (level_cluster_kernel): the same runs of small levels and the
// same ring codes as level_run_kernel, spread over a thread-block cluster of
// CC CTAs of 2^shift threads each (CC * 2^shift at least the run's widest
// level).  Position p of a level belongs to CTA p >> shift, whose ring holds
// the values its positions wrote in the last kRing levels (slot
// (level mod kRing) << shift | p mod 2^shift); a value another CTA wrote is
// read from that CTA's ring through distributed shared memory, and the
// cluster barrier replaces __syncthreads.  GB300 executes 2 FP64 FMAs per
// clock per SM, so a level of 512 rows with two or three entries each keeps
// one SM's FP64 pipe busy for ~500-800 cycles; eight SMs take an eighth of
// that.  Global values are read at L2 (ld.global.cg): they may have been
// written by another CTA, whose stores the cluster barrier's release/acquire
// orders but whose lines this SM's L1 could hold stale.  The arrive/wait pair
// is split around the next level's pattern fetch and the global store.  The
// per-row subtraction order is level_run_kernel's, so the results are equal.
template <typename T>
struct ClRing {
  T *local;             // this CTA's ring, kRing << shift values
  uint32_t rank, shift;
};

template <typename T>
__device__ __forceinline__ T cl_ring_read(uint32_t g, const ClRing<T> &rg) {
  const uint32_t p = g & (kCodeWidth - 1), e = (g >> kCodeShift) & (kRing - 1);
  const uint32_t owner = p >> rg.shift, slot = (e << rg.shift) | (p & ((1u << rg.shift) - 1));
  if (owner == rg.rank) return rg.local[slot];
  return cg::this_cluster().map_shared_rank(rg.local, owner)[slot];
}

template <typename T>
__device__ __forceinline__ T cl_read(int32_t code, const ClRing<T> &rg, const T *vec) {
  return code < 0 ? cl_ring_read<T>((uint32_t)~code, rg) : __ldcg(vec + code);
}

__device__ __forceinline__ void cluster_arrive_release() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void cluster_wait_acquire() {
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

template <typename T, int DE>
__device__ __forceinline__ void cl_level(uint32_t lev, uint32_t lev1, uint32_t pos,
                                         RunEntries<T> &ent, RunRow &row,
                                         const uint32_t *__restrict__ level_ptr,
                                         const uint32_t *__restrict__ row_index,
                                         const int32_t *__restrict__ xcode,
                                         const uint32_t *__restrict__ row_ptr,
                                         const int32_t *__restrict__ ecode,
                                         const T *__restrict__ vals, T *vec,
                                         const ClRing<T> &rg) {
  const RunRow r = ent.r;
  T x = T(0), y[kRunPre];
  if (r.row != kNoRow) x = r.xc >= 0 ? ent.xg : cl_ring_read<T>((uint32_t)~r.xc, rg);
#pragma unroll
  for (int k = 0; k < kRunPre; ++k) y[k] = r.jb + k < r.je ? cl_read<T>(ent.c[k], rg, vec) : T(0);
  T s = x;
  if (r.row != kNoRow) {
#pragma unroll
    for (int k = 0; k < kRunPre; ++k)
      if (r.jb + k < r.je) s -= y[k] * ent.v[k];
    for (uint32_t j = r.jb + kRunPre; j < r.je; ++j)
      s -= cl_read<T>(__ldg(ecode + j), rg, vec) * __ldg(vals + j);
    rg.local[((lev & (kRing - 1)) << rg.shift) | threadIdx.x] = s;
  }
  cluster_arrive_release();
  ent = run_fetch_entries<T, true>(row, ecode, vals, vec);
  row = run_fetch_row(lev + 2 * DE, lev1, level_ptr, row_index, xcode, row_ptr, pos);
  // read kRing levels later at the earliest, after at least one more barrier
  if (r.row != kNoRow) vec[r.row] = s;
  cluster_wait_acquire();
}

template <typename T, int DE, uint32_t NTMAX>
__global__ void __launch_bounds__(NTMAX)
    level_cluster_kernel(uint32_t lev0, uint32_t lev1, const uint32_t *__restrict__ level_ptr,
                         const uint32_t *__restrict__ row_index, const int32_t *__restrict__ xcode,
                         const uint32_t *__restrict__ row_ptr, const int32_t *__restrict__ ecode,
                         const T *__restrict__ vals, T *vec, const int *skip, uint32_t shift) {
  static_assert(DE >= 1 && DE < (int)kRing, "pipeline depth");
  extern __shared__ __align__(16) unsigned char ring_bytes[];
  if (skip && *skip) return;  // the same word for every CTA: the cluster leaves together
  const ClRing<T> rg{reinterpret_cast<T *>(ring_bytes), cg::this_cluster().block_rank(), shift};
  const uint32_t pos = (rg.rank << shift) | threadIdx.x;
  RunEntries<T> ents[DE];
  RunRow rows[DE];
#pragma unroll
  for (int k = 0; k < DE; ++k)
    ents[k] = run_fetch_entries<T, true>(
        run_fetch_row(lev0 + k, lev1, level_ptr, row_index, xcode, row_ptr, pos), ecode, vals,
        vec);
#pragma unroll
  for (int k = 0; k < DE; ++k)
    rows[k] = run_fetch_row(lev0 + DE + k, lev1, level_ptr, row_index, xcode, row_ptr, pos);
  for (uint32_t lev = lev0; lev < lev1; lev += DE) {
#pragma unroll
    for (int k = 0; k < DE; ++k) {
      if (lev + k >= lev1) break;  // uniform over the cluster
      cl_level<T, DE>(lev + k, lev1, pos, ents[k], rows[k], level_ptr, row_index, xcode, row_ptr,
                      ecode, vals, vec, rg);
    }
  }
  // every read of another CTA's ring came before the last barrier, so each
  // CTA may leave now
}

// Cluster size for runs of small levels: the largest of 16, 8 and 4 CTAs of
// 1024 threads (128 KB of ring each) that the device can co-schedule
// (occupancy query, once per precision), 0 if none.
template <typename T>
static int cluster_ctas() {
  static std::atomic<int> cached{-1};
  int v = cached.load(std::memory_order_relaxed);
  if (v >= 0) return v;
  v = 0;
  auto wide = level_cluster_kernel<T, 1, 1024>;
  auto deep = level_cluster_kernel<T, 4, 256>;
  const size_t wide_smem = (size_t)kRing * 1024 * sizeof(T);
  bool ok = cudaFuncSetAttribute(wide, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(deep, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
                cudaSuccess &&
            cudaFuncSetAttribute(wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)wide_smem) == cudaSuccess;
  for (int cc : {16, 8, 4}) {
    if (!ok) break;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cc);
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = wide_smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cc;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, wide, &cfg) == cudaSuccess && clusters > 0) {
      v = cc;
      break;
    }
  }
  (void)cudaGetLastError();
  cached.store(v, std::memory_order_relaxed);
  return v;
}

// One run of small levels [L, L1) on a cluster: position p of a level on CTA
// p >> shift, 2^shift threads a CTA (at least a warp), as few CTAs as cover
// the widest level.  CTAs of up to 256 threads fetch the pattern four levels
// ahead; wider ones one level ahead (registers).
template <typename T>
static void cluster_run(Backend &be, const Precond::Tri &tri, uint32_t L, uint32_t L1,
                        uint32_t widest, int cc, T *vec, const int *skip) {
  uint32_t shift = 5;
  while (((uint32_t)cc << shift) < widest) ++shift;
  const uint32_t ctas = std::max<uint32_t>(1, (widest + (1u << shift) - 1) >> shift);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(1u << shift);
  cfg.dynamicSmemBytes = ((size_t)kRing << shift) * sizeof(T);
  cfg.stream = be.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  auto kern = shift <= 8 ? level_cluster_kernel<T, 4, 256> : level_cluster_kernel<T, 1, 1024>;
  VCLGB_CUDA(cudaLaunchKernelEx(&cfg, kern, L, L1, tri.level_ptr.as<uint32_t>(),
                                tri.row_index.as<uint32_t>(), tri.xcode.as<int32_t>(),
                                tri.row_ptr.as<uint32_t>(), tri.ecode.as<int32_t>(),
                                tri.vals.as<T>(), vec, skip, shift));
}

template <typename X>
static void upload(Backend &be, DevBuf &dst, const std::vector<X> &src) {
  dst.alloc(std::max<size_t>(src.size(), 1) * sizeof(X), be.stream);
  if (!src.empty())
    VCLGB_CUDA(cudaMemcpyAsync(dst.ptr, src.data(), src.size() * sizeof(X),
                               cudaMemcpyHostToDevice, be.stream));
}

// The widest level a run may hold: a cluster's width where clusters can be
// launched, else a block's.
template <typename T>
static uint32_t run_width_for() {
  const int cc = cluster_ctas<T>();
  return cc > 0 ? (uint32_t)cc * 1024 : kRunLevel;
}

// Device copy of one triangle's level structure (pattern only): level
// pointers, level rows, per-level row pointers and columns, and the ring
// codes of its runs (plan_codes).
template <typename T>
static void tri_structure(Backend &be, const LevelPlan &pl, Precond::Tri &tri) {
  tri.levels = (uint32_t)(pl.level_ptr.size() - 1);
  tri.rows = pl.row_index.size();
  tri.nnz = pl.cols.size();
  tri.h_level_ptr = pl.level_ptr;
  tri.run_width = pl.run_width;
  tri.clusters = cluster_ctas<T>();
  if (tri.run_width) {
    upload(be, tri.ecode, pl.ecode);
    upload(be, tri.xcode, pl.xcode);
    VCLGB_CUDA(cudaFuncSetAttribute(level_run_kernel<T, kRunLevel, 1>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(kRingSlots * sizeof(T))));
    VCLGB_CUDA(cudaFuncSetAttribute(level_run_kernel<T, kRunLevel / 2, 4>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(kRingSlots * sizeof(T))));
  }
  upload(be, tri.level_ptr, pl.level_ptr);
  upload(be, tri.row_index, pl.row_index);
  upload(be, tri.row_ptr, pl.row_ptr);
  upload(be, tri.cols, pl.cols);
}

template <typename T>
static void ilu0_build(Backend &be, const Matrix &A, Precond &P) {
  const uint32_t n = A.rows;
  std::vector<uint32_t> rp(n + 1), ci(A.nnz);
  VCLGB_CUDA(cudaMemcpyAsync(rp.data(), A.row_ptr, rp.size() * 4, cudaMemcpyDeviceToHost, be.stream));
  if (A.nnz)
    VCLGB_CUDA(cudaMemcpyAsync(ci.data(), A.col_idx, ci.size() * 4, cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  // U's levels and codes are planned on a second host thread while this one
  // plans L, launches the factorisation and uploads L's structure
  const uint32_t rw = run_width_for<T>();
  LevelPlan U;
  std::exception_ptr u_error;
  std::thread u_planner([&]() {
    try {
      U = plan_levels(n, rp, ci, true, nullptr);
      plan_codes(U, n, rw);
    } catch (...) {
      u_error = std::current_exception();
    }
  });
  struct Join {
    std::thread &t;
    ~Join() {
      if (t.joinable()) t.join();
    }
  } join_u{u_planner};
  std::vector<uint32_t> levL;
  LevelPlan L = plan_levels(n, rp, ci, false, &levL);

  // factorisation order: rows grouped by their L level (ascending rows in a level)
  uint32_t maxlev = 0;
  for (uint32_t r = 0; r < n; ++r) maxlev = std::max(maxlev, levL[r]);
  std::vector<uint32_t> lvl_cnt(maxlev + 2, 0);
  for (uint32_t r = 0; r < n; ++r) lvl_cnt[levL[r]] += 1;
  std::vector<uint32_t> lvl_off(maxlev + 2, 0);
  for (uint32_t e = 1; e <= maxlev + 1; ++e) lvl_off[e] = lvl_off[e - 1] + lvl_cnt[e - 1];
  std::vector<uint32_t> order(n), cur(lvl_off);
  for (uint32_t r = 0; r < n; ++r) order[cur[levL[r]]++] = r;

  P.lu.alloc(std::max<uint64_t>(A.nnz, 1) * sizeof(T), be.stream);
  if (A.nnz)
    VCLGB_CUDA(cudaMemcpyAsync(P.lu.ptr, A.values, A.nnz * sizeof(T), cudaMemcpyDeviceToDevice,
                               be.stream));
  DevBuf d_order, d_off;
  upload(be, d_order, order);
  upload(be, d_off, lvl_off);
  for (uint32_t e = 1; e <= maxlev;) {
    uint32_t c = lvl_cnt[e];
    if (c <= kFactorRun) {  // a run of small levels: one block
      uint32_t e1 = e + 1;
      while (e1 <= maxlev && lvl_cnt[e1] <= kFactorRun) ++e1;
      ilu0_run_kernel<T><<<1, kFactorRun, 0, be.stream>>>(
          e, e1, d_off.as<uint32_t>(), d_order.as<uint32_t>(), A.row_ptr, A.col_idx,
          P.lu.as<T>());
      be.launches++;
      e = e1;
      continue;
    }
    int g = waves_grid(be, 128, 16, c);
    ilu0_level_kernel<T><<<g, 128, 0, be.stream>>>(c, d_order.as<uint32_t>() + lvl_off[e],
                                                   A.row_ptr, A.col_idx, P.lu.as<T>());
    be.launches++;
    ++e;
  }
  VCLGB_CHECK_LAUNCH();
  // U diagonal of the factors
  {
    Matrix tmp;
    tmp.format = VCLGB_CSR;
    tmp.prec = A.prec;
    tmp.rows = n;
    tmp.cols = n;
    tmp.nnz = A.nnz;
    tmp.row_ptr = A.row_ptr;
    tmp.col_idx = A.col_idx;
    tmp.values = P.lu.ptr;
    extract_diag(be, tmp, P.diag, false);
  }
  auto fill_tri = [&](LevelPlan &pl, Precond::Tri &tri, bool upper) {
    tri_structure<T>(be, pl, tri);
    DevBuf src;
    upload(be, src, pl.src);
    tri.vals.alloc(std::max<uint64_t>(tri.nnz, 1) * sizeof(T), be.stream);
    if (tri.nnz) {
      int g = waves_grid(be, 256, 8, tri.rows);
      level_vals_kernel<T><<<g, 256, 0, be.stream>>>(
          tri.rows, tri.row_index.as<uint32_t>(), tri.row_ptr.as<uint32_t>(), src.as<uint32_t>(),
          P.lu.as<T>(), upper ? P.diag.as<T>() : nullptr, tri.vals.as<T>());
      be.launches++;
      VCLGB_CHECK_LAUNCH();
    }
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));  // src freed after use
  };
  plan_codes(L, n, rw);
  fill_tri(L, P.L, false);
  u_planner.join();
  if (u_error) std::rethrow_exception(u_error);
  fill_tri(U, P.U, true);
}

std::unique_ptr<Precond> ilu0_create(Backend &be, const Matrix &A, bool level_scheduling) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "ilu0_precond is built from CSR");
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "ILU0 needs a square matrix");
  auto P = std::make_unique<Precond>();
  P->kind = 2;
  P->prec = A.prec;
  P->rows = A.rows;
  P->nnz = A.nnz;
  P->row_ptr = A.row_ptr;
  P->col_idx = A.col_idx;
  // the device apply is level-scheduled either way: without level scheduling the
  // reference copies the vector to the host and solves sequentially
  // (ilu0.hpp:229-236); both orders give the same substitution up to rounding
  P->level_scheduling = level_scheduling;
  if (A.prec == VCLGB_FLOAT64)
    ilu0_build<double>(be, A, *P);
  else
    ilu0_build<float>(be, A, *P);
  return P;
}

// ---------------------------------------------------------------------------
// block_ilu_precond<compressed_matrix, ilu0_tag> (linalg/detail/ilu/block_ilu.hpp:
// 322-365, extract_block_matrix :69-113): ILU0 of A restricted to its diagonal
// blocks.  The reference factorises every block on the host and solves block
// by block; here the block-diagonal part of A (an entry whose column lies
// outside its row's block is dropped, order kept) goes through the device
// ILU0 above.  A row's elimination never leaves its block, so the factors are
// the reference's per-block factors side by side, bit for bit, and the level
// schedule runs all blocks at once.  `starts` holds the blocks' first rows and
// n at the end; the blocks tile [0, n).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void block_of_row(uint32_t r, const uint32_t *starts, uint32_t nb,
                                             uint32_t &lo, uint32_t &hi) {
  uint32_t a = 0, b = nb;  // last block whose start is <= r (empty blocks skipped)
  while (a + 1 < b) {
    const uint32_t m = (a + b) / 2;
    if (starts[m] <= r) a = m; else b = m;
  }
  lo = starts[a];
  hi = starts[a + 1];
}

__global__ void block_count_kernel(uint32_t n, const uint32_t *__restrict__ rp,
                                   const uint32_t *__restrict__ ci,
                                   const uint32_t *__restrict__ starts, uint32_t nb,
                                   uint32_t *cnt) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x) {
    uint32_t lo, hi, c = 0;
    block_of_row((uint32_t)r, starts, nb, lo, hi);
    for (uint32_t j = rp[r]; j < rp[r + 1]; ++j) c += ci[j] >= lo && ci[j] < hi;
    cnt[r] = c;
  }
}

template <typename W>
__global__ void block_fill_kernel(uint32_t n, const uint32_t *__restrict__ rp,
                                  const uint32_t *__restrict__ ci, const W *__restrict__ v,
                                  const uint32_t *__restrict__ starts, uint32_t nb,
                                  const uint32_t *__restrict__ brp, uint32_t *bci, W *bv) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x) {
    uint32_t lo, hi, k = brp[r];
    block_of_row((uint32_t)r, starts, nb, lo, hi);
    for (uint32_t j = rp[r]; j < rp[r + 1]; ++j)
      if (ci[j] >= lo && ci[j] < hi) {
        bci[k] = ci[j];
        bv[k] = v[j];
        ++k;
      }
  }
}

std::unique_ptr<Precond> block_ilu0_create(Backend &be, const Matrix &A, uint32_t num_blocks,
                                           const uint32_t *h_bounds) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "block_ilu_precond is built from CSR");
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "block ILU needs a square matrix");
  require(num_blocks > 0, VCLGB_INVALID_ARGUMENT, "block ILU needs at least one block");
  const uint32_t n = A.rows;
  std::vector<uint32_t> starts(num_blocks + 1);
  if (!h_bounds) {
    // the reference's default split (block_ilu.hpp:325-333)
    for (uint32_t i = 0; i <= num_blocks; ++i)
      starts[i] = (uint32_t)(((uint64_t)i * n) / num_blocks);
  } else {
    std::vector<std::pair<uint32_t, uint32_t>> b(num_blocks);
    for (uint32_t i = 0; i < num_blocks; ++i) b[i] = {h_bounds[2 * i], h_bounds[2 * i + 1]};
    std::sort(b.begin(), b.end());
    // rows outside every block would be divided by a zero D in the reference's
    // apply; blocks that overlap would be solved twice: both are rejected
    uint32_t at = 0;
    for (uint32_t i = 0; i < num_blocks; ++i) {
      require(b[i].first == at && b[i].second >= b[i].first, VCLGB_INVALID_ARGUMENT,
              "block boundaries must tile [0, rows) without gaps or overlaps");
      starts[i] = at;
      at = b[i].second;
    }
    require(at == n, VCLGB_INVALID_ARGUMENT,
            "block boundaries must tile [0, rows) without gaps or overlaps");
    starts[num_blocks] = n;
  }
  auto m = std::make_unique<Matrix>();
  m->format = VCLGB_CSR;
  m->prec = A.prec;
  m->rows = m->cols = n;
  m->own_row_ptr.alloc(((size_t)n + 1) * 4, be.stream);
  if (n) {
    DevBuf d_starts, cnt(((size_t)n) * 4, be.stream);
    upload(be, d_starts, starts);
    const int g = waves_grid(be, 256, 8, n);
    block_count_kernel<<<g, 256, 0, be.stream>>>(n, A.row_ptr, A.col_idx,
                                                 d_starts.as<uint32_t>(), num_blocks,
                                                 cnt.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    m->nnz = extern_scan_u32(be, cnt.as<uint32_t>(), n, m->own_row_ptr.as<uint32_t>());
    m->own_col_idx.alloc(std::max<uint64_t>(m->nnz, 1) * 4, be.stream);
    m->own_values.alloc(std::max<uint64_t>(m->nnz, 1) * A.vsize(), be.stream);
    if (A.vsize() == 8)
      block_fill_kernel<uint64_t><<<g, 256, 0, be.stream>>>(
          n, A.row_ptr, A.col_idx, static_cast<const uint64_t *>(A.values),
          d_starts.as<uint32_t>(), num_blocks, m->own_row_ptr.as<uint32_t>(),
          m->own_col_idx.as<uint32_t>(), m->own_values.as<uint64_t>());
    else
      block_fill_kernel<uint32_t><<<g, 256, 0, be.stream>>>(
          n, A.row_ptr, A.col_idx, static_cast<const uint32_t *>(A.values),
          d_starts.as<uint32_t>(), num_blocks, m->own_row_ptr.as<uint32_t>(),
          m->own_col_idx.as<uint32_t>(), m->own_values.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));  // d_starts/cnt freed after use
  } else {
    VCLGB_CUDA(cudaMemsetAsync(m->own_row_ptr.ptr, 0, 4, be.stream));
    m->own_col_idx.alloc(4, be.stream);
    m->own_values.alloc(8, be.stream);
  }
  m->row_ptr = m->own_row_ptr.as<uint32_t>();
  m->col_idx = m->own_col_idx.as<uint32_t>();
  m->values = m->own_values.ptr;
  auto P = ilu0_create(be, *m, true);
  P->blocks = num_blocks;
  P->owned = std::move(m);
  return P;
}

// Runs whose levels hold at most kRunLevel / 2 rows take one block (a level
// costs less there than the cluster barrier, ~0.42 us on GB300); wider runs a
// cluster where one can be launched, else one block of kRunLevel threads.
template <typename T>
static void tri_apply(Backend &be, const Precond::Tri &tri, T *vec, const int *skip) {
  for (uint32_t L = 0; L < tri.levels;) {
    const uint32_t r0 = tri.h_level_ptr[L], r1 = tri.h_level_ptr[L + 1];
    const uint32_t L1 = run_end(tri.h_level_ptr, L, tri.run_width);
    if (L1 > L) {
      const size_t smem = kRingSlots * sizeof(T);
      const uint32_t widest = widest_level(tri.h_level_ptr, L, L1);
      if (widest > kRunLevel / 2 && tri.clusters > 0)
        cluster_run<T>(be, tri, L, L1, widest, tri.clusters, vec, skip);
      else if (widest <= kRunLevel / 2)
        level_run_kernel<T, kRunLevel / 2, 4><<<1, kRunLevel / 2, smem, be.stream>>>(
            L, L1, tri.level_ptr.as<uint32_t>(), tri.row_index.as<uint32_t>(),
            tri.xcode.as<int32_t>(), tri.row_ptr.as<uint32_t>(), tri.ecode.as<int32_t>(),
            tri.vals.as<T>(), vec, skip);
      else
        level_run_kernel<T, kRunLevel, 1><<<1, kRunLevel, smem, be.stream>>>(
            L, L1, tri.level_ptr.as<uint32_t>(), tri.row_index.as<uint32_t>(),
            tri.xcode.as<int32_t>(), tri.row_ptr.as<uint32_t>(), tri.ecode.as<int32_t>(),
            tri.vals.as<T>(), vec, skip);
      be.launches++;
      L = L1;
      continue;
    }
    int g = waves_grid(be, 128, 16, r1 - r0);
    level_substitute_kernel<T><<<g, 128, 0, be.stream>>>(
        r0, r1, tri.row_index.as<uint32_t>(), tri.row_ptr.as<uint32_t>(), tri.cols.as<uint32_t>(),
        tri.vals.as<T>(), vec, skip);
    be.launches++;
    ++L;
  }
  VCLGB_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// CSR triangular solves: inplace_solve(A, vec, tag) and inplace_solve(trans(A),
// vec, tag) (linalg/host_based/sparse_matrix_operations.hpp:537-1090; the CUDA
// backend runs them as one block of 128 threads, linalg/cuda/
// sparse_matrix_operations.hpp:780-1008).  The rows of the tag's strict
// triangle are put in levels as the ILU0 substitution's are (a row's level is
// one more than the deepest level among its columns), so each level is one
// parallel step: runs of small levels in one block (level_run_kernel), wide
// levels grid-wide.  The non-unit forms divide the right-hand side by the
// diagonal first and substitute with the entries divided by their row's
// diagonal (x_r = b_r/d_r - sum (a_rc/d_r) x_c, as the ILU0 U solve does);
// the unit forms use the entries as they are.  trans(A) runs the same on the
// pattern of A^T (transpose map of the adjoint), its entries read from A.
// The level structure depends on the pattern only and is cached on the
// matrix; the values are gathered again at every call.
// ---------------------------------------------------------------------------
struct TriSolvePlan {
  Precond::Tri tri;
  DevBuf src;  // entry of A behind each level entry
  DevBuf diag;
};

template <typename T>
static void csr_inplace_solve_t(Backend &be, Matrix &A, int tag, bool trans, T *vec) {
  const bool upper = tag == 1 || tag == 3, unit = tag >= 2;
  const uint32_t n = A.rows;
  auto &slot = A.tri_plan[(upper ? 1 : 0) | (trans ? 2 : 0)];
  if (!slot) {
    auto plan = std::make_shared<TriSolvePlan>();
    std::vector<uint32_t> rp(n + 1), ci(A.nnz), map;
    if (trans) {
      DevBuf trp, tci, m;
      csr_transpose_pattern(be, A.rows, A.cols, A.nnz, A.row_ptr, A.col_idx, trp, tci, m);
      map.resize(A.nnz);
      VCLGB_CUDA(cudaMemcpyAsync(rp.data(), trp.ptr, rp.size() * 4, cudaMemcpyDeviceToHost,
                                 be.stream));
      if (A.nnz) {
        VCLGB_CUDA(cudaMemcpyAsync(ci.data(), tci.ptr, ci.size() * 4, cudaMemcpyDeviceToHost,
                                   be.stream));
        VCLGB_CUDA(cudaMemcpyAsync(map.data(), m.ptr, map.size() * 4, cudaMemcpyDeviceToHost,
                                   be.stream));
      }
      VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    } else {
      VCLGB_CUDA(cudaMemcpyAsync(rp.data(), A.row_ptr, rp.size() * 4, cudaMemcpyDeviceToHost,
                                 be.stream));
      if (A.nnz)
        VCLGB_CUDA(cudaMemcpyAsync(ci.data(), A.col_idx, ci.size() * 4, cudaMemcpyDeviceToHost,
                                   be.stream));
      VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    }
    LevelPlan pl = plan_levels(n, rp, ci, upper, nullptr);
    plan_codes(pl, n, run_width_for<T>());
    if (trans)
      for (auto &k : pl.src) k = map[k];
    tri_structure<T>(be, pl, plan->tri);
    upload(be, plan->src, pl.src);
    plan->tri.vals.alloc(std::max<uint64_t>(plan->tri.nnz, 1) * sizeof(T), be.stream);
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));  // host plan freed after the uploads
    slot = std::move(plan);
  }
  TriSolvePlan &P = *slot;
  if (!unit) extract_diag(be, A, P.diag, false);
  if (P.tri.nnz) {
    const int g = waves_grid(be, 256, 8, P.tri.rows);
    level_vals_kernel<T><<<g, 256, 0, be.stream>>>(
        P.tri.rows, P.tri.row_index.as<uint32_t>(), P.tri.row_ptr.as<uint32_t>(),
        P.src.as<uint32_t>(), static_cast<const T *>(A.values), unit ? nullptr : P.diag.as<T>(),
        P.tri.vals.as<T>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  }
  if (!unit && n) {
    const int g = waves_grid(be, 256, 8, n);
    div_kernel<T><<<g, 256, 0, be.stream>>>(n, vec, P.diag.as<T>(), nullptr);
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  }
  tri_apply<T>(be, P.tri, vec, nullptr);
}

void csr_inplace_solve(Backend &be, Matrix &A, int tag, bool trans, void *d_vec) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "inplace_solve takes a CSR matrix");
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "inplace_solve needs a square matrix");
  require(tag >= 0 && tag <= 3, VCLGB_INVALID_ARGUMENT,
          "tag must be 0 lower, 1 upper, 2 unit_lower or 3 unit_upper");
  if (A.prec == VCLGB_FLOAT64)
    csr_inplace_solve_t<double>(be, A, tag, trans, static_cast<double *>(d_vec));
  else
    csr_inplace_solve_t<float>(be, A, tag, trans, static_cast<float *>(d_vec));
}

void precond_apply(Backend &be, const Precond &P, void *d_vec, const int *skip_flag) {
  if (P.kind == 3 || P.kind == 4) {
    chow_patel_apply(be, P, d_vec, skip_flag);
    return;
  }
  if (P.kind == 1) {
    int g = waves_grid(be, 256, 8, P.rows);
    if (P.prec == VCLGB_FLOAT64)
      div_kernel<double><<<g, 256, 0, be.stream>>>(P.rows, static_cast<double *>(d_vec),
                                                   P.diag.as<double>(), skip_flag);
    else
      div_kernel<float><<<g, 256, 0, be.stream>>>(P.rows, static_cast<float *>(d_vec),
                                                  P.diag.as<float>(), skip_flag);
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    return;
  }
  // ILU0: L levels, divide by the U diagonal, U levels (ilu0.hpp:213-226)
  int g = waves_grid(be, 256, 8, P.rows);
  if (P.prec == VCLGB_FLOAT64) {
    tri_apply<double>(be, P.L, static_cast<double *>(d_vec), skip_flag);
    div_kernel<double><<<g, 256, 0, be.stream>>>(P.rows, static_cast<double *>(d_vec),
                                                 P.diag.as<double>(), skip_flag);
    be.launches++;
    tri_apply<double>(be, P.U, static_cast<double *>(d_vec), skip_flag);
  } else {
    tri_apply<float>(be, P.L, static_cast<float *>(d_vec), skip_flag);
    div_kernel<float><<<g, 256, 0, be.stream>>>(P.rows, static_cast<float *>(d_vec),
                                                P.diag.as<float>(), skip_flag);
    be.launches++;
    tri_apply<float>(be, P.U, static_cast<float *>(d_vec), skip_flag);
  }
  VCLGB_CHECK_LAUNCH();
}

}  // namespace vclgb
