// noalloc.cu -- HYB SpMV that allocates no memory (no counterpart in the reference).
//
// The regular HYB product allocates a small carry buffer per call for the
// warp-segmented reduction of the COO tail, and the engine's matrix objects
// allocate when they are built.  This variant takes the hyb_matrix arrays
// exactly as the reference stores them (ELL part, CSR tail) and keeps the
// carries in a fixed file-scope device array, so a call performs no
// allocation of any kind.  The tail entry's row is found by binary search in
// the tail row_ptr instead of a COO row array.
#include <atomic>
#include <mutex>

#include "spmv.cuh"

namespace vclgb {

// Largest tail the fixed scratch serves: 2^23 entries = 32,768 chunks of 256,
// two carries (row u32 + value f64) per chunk = 768 KiB per device.
constexpr uint64_t kNoAllocMaxTail = 1ull << 23;
constexpr size_t kNoAllocChunks = (kNoAllocMaxTail + kTailChunk - 1) / kTailChunk;
constexpr size_t kNoAllocRowBytes = 2 * kNoAllocChunks * sizeof(uint32_t);
constexpr size_t kNoAllocBytes = kNoAllocRowBytes + 2 * kNoAllocChunks * sizeof(double);

// Shared by every call on a device; it keeps the last call's contents.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct NoAllocDevice {
  void *scratch = nullptr;  // device address of g_noalloc_scratch on this device
  int num_sms = 0;
  // set (release) once scratch and num_sms are filled in; later calls read it
  // (acquire) without taking the set-up lock
  std::atomic<bool> ready{false};
};
static NoAllocDevice g_noalloc_dev[64];
static std::mutex g_noalloc_mutex;

// row of tail entry k: the last r with trp[r] <= k, searched in [lo, hi]
__device__ __forceinline__ uint32_t tail_row_of(const uint32_t *__restrict__ trp, uint32_t lo,
                                                uint32_t hi, uint64_t k) {
  while (lo < hi) {
    uint32_t mid = lo + (hi - lo + 1) / 2;
    if ((uint64_t)__ldg(trp + mid) <= k) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// The tail kernel of spmv.cuh with rows taken from the CSR tail row_ptr: per
// chunk, lane 0 finds the rows of its first and last entry; every lane then
// searches its own row inside that range.
template <typename T>
__global__ void __launch_bounds__(kSpmvThreads)
    hyb_tail_csr_kernel(uint32_t rows, uint64_t tnnz, const uint32_t *__restrict__ trp,
                        const uint32_t *__restrict__ tcol, const T *__restrict__ tval,
                        const T *__restrict__ x, T alpha, T *y, uint32_t *carry_row,
                        T *carry_val) {
  const uint32_t INV = 0xffffffffu;
  const uint32_t lane = threadIdx.x & 31;
  const size_t nchunks = (tnnz + kTailChunk - 1) / kTailChunk;
  const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t ch = warp; ch < nchunks; ch += nwarps) {
    const size_t c0 = ch * kTailChunk;
    const size_t c1 = c0 + kTailChunk < tnnz ? c0 + kTailChunk : tnnz;
    uint32_t lo = 0, hi = 0;
    if (lane == 0) {
      lo = tail_row_of(trp, 0, rows - 1, c0);
      hi = tail_row_of(trp, lo, rows - 1, c1 - 1);
    }
    lo = __shfl_sync(0xffffffffu, lo, 0);
    hi = __shfl_sync(0xffffffffu, hi, 0);
    const uint32_t first_row = lo, last_row = hi;
    T run = 0;
    uint32_t run_row = INV;
    for (size_t k0 = c0; k0 < c1; k0 += 32) {
      const size_t k = k0 + lane;
      const bool ok = k < c1;
      const uint32_t r = ok ? tail_row_of(trp, lo, hi, k) : INV;
      T p = ok ? __ldg(tval + k) * __ldg(x + __ldg(tcol + k)) : T(0);
      if (lane == 0 && r == run_row) p += run;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        T q = __shfl_up_sync(0xffffffffu, p, o);
        uint32_t qr = __shfl_up_sync(0xffffffffu, r, o);
        if ((int)lane >= o && qr == r) p += q;
      }
      uint32_t nr = __shfl_down_sync(0xffffffffu, r, 1);
      if (lane == 31) nr = (k + 1 < c1) ? tail_row_of(trp, lo, hi, k + 1) : INV;
      if (ok && nr != r) {
        if (r == first_row) {
          carry_row[2 * ch] = r;
          carry_val[2 * ch] = p;
        } else if (r == last_row) {
          carry_row[2 * ch + 1] = r;
          carry_val[2 * ch + 1] = p;
        } else {
          y[r] += alpha * p;
        }
      }
      const int lastlane = (int)((c1 - k0 < 32 ? c1 - k0 : 32) - 1);
      run = __shfl_sync(0xffffffffu, p, lastlane);
      run_row = __shfl_sync(0xffffffffu, r, lastlane);
    }
    if (lane == 0 && first_row == last_row) carry_row[2 * ch + 1] = INV;
  }
}

template <typename T, int MODE>
static void ell_part(cudaStream_t s, int grid, uint32_t rows, uint32_t width,
                     const uint32_t *coords, const T *elems, const T *x, T alpha, T beta, T *y) {
  EpiAxpbyM<T, MODE> e{alpha, beta, y, 0, 1};
#define VCLGB_NA_ELL(W)                                                                      \
  ell_kernel<W, T, EpiAxpbyM<T, MODE>><<<grid, kSpmvThreads, 0, s>>>(rows, width, coords,   \
                                                                     elems, x, 0, 1, e,      \
                                                                     nullptr, nullptr)
  switch (width) {
    case 1: VCLGB_NA_ELL(1); break;
    case 2: VCLGB_NA_ELL(2); break;
    case 3: VCLGB_NA_ELL(3); break;
    case 4: VCLGB_NA_ELL(4); break;
    case 5: VCLGB_NA_ELL(5); break;
    case 6: VCLGB_NA_ELL(6); break;
    case 7: VCLGB_NA_ELL(7); break;
    case 8: VCLGB_NA_ELL(8); break;
    default: VCLGB_NA_ELL(0); break;
  }
#undef VCLGB_NA_ELL
}

template <typename T>
static vclgbStatus hyb_noalloc(cudaStream_t s, const NoAllocDevice &dev, uint32_t rows,
                               uint32_t width, const uint32_t *coords, const void *elems,
                               const uint32_t *trp, const uint32_t *tcol, const void *tval,
                               uint64_t tnnz, double alpha_d, const void *xv, double beta_d,
                               void *yv) {
  const T alpha = (T)alpha_d, beta = (T)beta_d;
  const T *x = static_cast<const T *>(xv);
  T *y = static_cast<T *>(yv);
  int per_sm = 8;
  size_t full = (size_t)dev.num_sms * per_sm;
  size_t need = ((size_t)rows + kSpmvThreads - 1) / kSpmvThreads;
  int grid = (int)std::max<size_t>(1, std::min(need, full));
  with_axpby_mode(alpha, beta, [&](auto mode) {
    ell_part<T, decltype(mode)::value>(s, grid, rows, width, coords,
                                       static_cast<const T *>(elems), x, alpha, beta, y);
  });
  if (tnnz > 0) {
    const size_t nchunks = (tnnz + kTailChunk - 1) / kTailChunk;
    uint32_t *carry_row = static_cast<uint32_t *>(dev.scratch);
    T *carry_val = reinterpret_cast<T *>(static_cast<unsigned char *>(dev.scratch) +
                                         kNoAllocRowBytes);
    int g = (int)std::max<size_t>(1, std::min((nchunks * 32 + kSpmvThreads - 1) / kSpmvThreads,
                                              full));
    hyb_tail_csr_kernel<T><<<g, kSpmvThreads, 0, s>>>(rows, tnnz, trp, tcol,
                                                      static_cast<const T *>(tval), x, alpha, y,
                                                      carry_row, carry_val);
    int g2 = (int)((nchunks + 255) / 256);
    hyb_tail_fixup<T><<<g2, 256, 0, s>>>(nchunks, carry_row, carry_val, alpha, y, 0, 1,
                                         nullptr);
  }
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? VCLGB_SUCCESS : VCLGB_CUDA_ERROR;
}

}  // namespace vclgb

using namespace vclgb;

extern "C" VCLGB_API vclgbStatus vclgbHybSpmvNoAlloc(
    void *cuda_stream, vclgbPrecision prec, uint32_t rows, uint32_t ell_width,
    const uint32_t *d_ell_coords, const void *d_ell_elems, const uint32_t *d_tail_row_ptr,
    const uint32_t *d_tail_cols, const void *d_tail_vals, uint64_t tail_nnz, double alpha,
    const void *d_x, double beta, void *d_y) {
  if (prec != VCLGB_FLOAT32 && prec != VCLGB_FLOAT64) return VCLGB_INVALID_ARGUMENT;
  if (tail_nnz > kNoAllocMaxTail) return VCLGB_INVALID_ARGUMENT;  // beyond the fixed scratch
  if (rows == 0) return VCLGB_SUCCESS;
  if (!d_x || !d_y || (ell_width && (!d_ell_coords || !d_ell_elems)) ||
      (tail_nnz && (!d_tail_row_ptr || !d_tail_cols || !d_tail_vals)))
    return VCLGB_INVALID_ARGUMENT;
  // an error left pending by an earlier call of the caller's is theirs to
  // read: it is neither cleared nor reported as this call's, and nothing runs
  if (cudaPeekAtLastError() != cudaSuccess) return VCLGB_CUDA_ERROR;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return VCLGB_CUDA_ERROR;
  NoAllocDevice &d = g_noalloc_dev[dev];
  if (!d.ready.load(std::memory_order_acquire)) {
    // one-time per-device set-up with this device current: the device address
    // of the scratch array (the host-side symbol is not a device address)
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!d.ready.load(std::memory_order_relaxed)) {
      void *ptr = nullptr;
      if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr)
        return VCLGB_CUDA_ERROR;
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return VCLGB_CUDA_ERROR;
      d.scratch = ptr;
      d.num_sms = sms;
      d.ready.store(true, std::memory_order_release);
    }
  }
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (prec == VCLGB_FLOAT64)
    return hyb_noalloc<double>(s, d, rows, ell_width, d_ell_coords, d_ell_elems, d_tail_row_ptr,
                               d_tail_cols, d_tail_vals, tail_nnz, alpha, d_x, beta, d_y);
  return hyb_noalloc<float>(s, d, rows, ell_width, d_ell_coords, d_ell_elems, d_tail_row_ptr,
                            d_tail_cols, d_tail_vals, tail_nnz, alpha, d_x, beta, d_y);
}
