// vclgb_internal.hpp -- shared host/device definitions of the GB300 sparse engine.
#pragma once

#include <cuda/atomic>
#include <cuda_runtime.h>
#include <atomic>
#include <initializer_list>
#include <stdint.h>

#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/vclgb.h"

namespace vclgb {

// ---------------------------------------------------------------------------
// errors: every C entry point catches these and turns them into a status.
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  vclgbStatus status;
  Error(vclgbStatus s, const std::string &m) : std::runtime_error(m), status(s) {}
};

#define VCLGB_CUDA(call)                                                                  \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      if (e_ == cudaErrorMemoryAllocation)                                                \
        throw ::vclgb::Error(VCLGB_OUT_OF_MEMORY, std::string(#call) + ": " +             \
                                                      cudaGetErrorString(e_));            \
      throw ::vclgb::Error(VCLGB_CUDA_ERROR,                                              \
                           std::string(#call) + ": " + cudaGetErrorString(e_));           \
    }                                                                                     \
  } while (0)

#define VCLGB_CHECK_LAUNCH() VCLGB_CUDA(cudaGetLastError())

inline void require(bool ok, vclgbStatus s, const char *msg) {
  if (!ok) throw Error(s, msg);
}

// ---------------------------------------------------------------------------
// device memory owned by the engine (stream-ordered pool allocations)
// ---------------------------------------------------------------------------
// Set (by FreesAfterDeviceSync) while a long-lived object is destroyed after
// cudaDeviceSynchronize: its buffers are then freed on the legacy default
// stream, which always exists, instead of the stream they were allocated on
// (which the caller may have destroyed since).
inline thread_local bool g_frees_after_device_sync = false;
struct FreesAfterDeviceSync {
  FreesAfterDeviceSync() { g_frees_after_device_sync = true; }
  ~FreesAfterDeviceSync() { g_frees_after_device_sync = false; }
};

struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  bool owned = true;  // false: the caller's array, never freed here
  DevBuf() = default;
  DevBuf(size_t b, cudaStream_t s) { alloc(b, s); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept { *this = std::move(o); }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) {
      release();
      ptr = o.ptr; bytes = o.bytes; stream = o.stream; owned = o.owned;
      o.ptr = nullptr; o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t b, cudaStream_t s) {
    release();
    stream = s;
    bytes = b;
    owned = true;
    if (b) VCLGB_CUDA(cudaMallocAsync(&ptr, b, s));
  }
  // wrap an existing device array (the reference's own buffers)
  void borrow(const void *p, size_t b) {
    release();
    ptr = const_cast<void *>(p);
    bytes = b;
    owned = false;
  }
  void release() noexcept {
    if (ptr && owned) cudaFreeAsync(ptr, g_frees_after_device_sync ? cudaStreamLegacy : stream);
    ptr = nullptr;
    bytes = 0;
    owned = true;
  }
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

// ---------------------------------------------------------------------------
// backend
// ---------------------------------------------------------------------------
struct Backend {
  int device = 0;
  int num_sms = 152;
  int max_threads_per_sm = 2048;
  size_t max_smem_per_block = 48 * 1024;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // a stream of the backend's own that vclgbBackendSetStream replaced: kept
  // until the backend is destroyed, because buffers allocated on it free on it
  cudaStream_t retired_stream = nullptr;
  std::string last_error;
  uint64_t launches = 0;
  // pinned host words the solvers read (status, loop trips); in the
  // host-polled mode (kernel timing, PDL) two chunks
  // in flight; the events mark when each status copy has landed
  int *host_flags = nullptr;
  cudaEvent_t poll_ev[2] = {nullptr, nullptr};
  // persistent reduction scratch for the vector reductions
  DevBuf red_partials;
  DevBuf red_counter;
  // trip counter of the solvers' device-side loops
  DevBuf loop_trips;
  // the buffers above follow the backend to a new stream, and are released
  // before the backend's own stream is destroyed
  void adopt_stream(cudaStream_t s) {
    for (DevBuf *b : {&red_partials, &red_counter, &loop_trips}) b->stream = s;
  }
  void release_buffers() {
    for (DevBuf *b : {&red_partials, &red_counter, &loop_trips}) b->release();
  }
  // kernel timing (off by default): every SpMV phase and fused vector pass is
  // bracketed by a pair of CUDA events, recorded as event nodes when the
  // launches are captured into a graph; durations (ms) by kind
  bool timing = false;
  std::vector<cudaEvent_t> tev;   // event pool, pairs (2k, 2k+1)
  std::vector<int> tev_kind;      // kind of pair k: 0 SpMV, 1 vector pass
  size_t tev_used = 0;            // events recorded since the last collection
  std::vector<float> times[2];
  // programmatic dependent launch for the solver kernels (off unless the
  // environment sets VCLGB_PDL=1): a kernel's blocks may start while the
  // previous kernel on the stream finishes, and wait for it on the device.
  // Measured on the 128^3 CG iteration (SpMV phase + update, graph-captured):
  // 78.1 us without, 79.6 us with -- the serial tail of each kernel's
  // last-block reduction is not hidden by starting the next kernel early.
  bool pdl = false;
  // L2 persisting access window put on every kernel launched through
  // launch_kernel (num_bytes 0: none); open only inside an L2Persist scope
  cudaAccessPolicyWindow l2_window = {};
  // the device's persisting-L2 limit, largest window and L2 size (read once)
  long l2_persist_max = -1, l2_window_max = 0, l2_bytes = 0;
};

// Launches kern<<<grid, block, smem, be.stream>>>(args...), with programmatic
// dependent launch when the backend allows it.  Every kernel launched through
// here calls pdl_wait() before it reads anything the previous kernel on the
// stream may write (without the attribute that wait returns at once).
template <typename... KArgs, typename... Args>
inline void launch_kernel(Backend &be, void (*kern)(KArgs...), int grid, int block, size_t smem,
                          Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = be.stream;
  cudaLaunchAttribute attr[2];
  unsigned na = 0;
  if (be.pdl) {
    attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
  }
  if (be.l2_window.num_bytes) {
    attr[na].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[na].val.accessPolicyWindow = be.l2_window;
    ++na;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  VCLGB_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
}

// Keeps a large solve's vectors resident in L2 while its matrix streams
// through it: the launches inside the scope carry an access-policy window over
// the leading part of the vectors that the set-aside holds, whose hits persist
// (misses stream), backed by a persisting set-aside of the context's L2.  Only
// where the vectors are large (32 MB or more), vectors and matrix together
// exceed L2, and the set-aside holds at least half of the vectors; the
// set-aside is a limit of the calling context, and the scope puts back the
// caller's value on exit, after the stream has drained and the persisting
// lines are released.
constexpr size_t kL2PersistMin = 32u << 20;

// The persisting set-aside is a limit of the device's context, shared by every
// solve of the process: the first scope to open saves the caller's value, a
// concurrent one may only raise it, and the last to close releases the
// persisting lines and puts the saved value back.
struct L2SetAside {
  std::mutex mu;
  int active = 0;
  size_t saved = 0, current = 0;
};
inline L2SetAside &l2_set_aside(int device) {
  static L2SetAside per_device[64];
  return per_device[device & 63];
}

struct L2Persist {
  Backend &be;
  bool on = false;
  L2Persist(Backend &b, void *base, size_t bytes, size_t other_bytes) : be(b) {
    if (bytes < kL2PersistMin) return;
    if (be.l2_persist_max < 0) {
      int pm = 0, wm = 0, l2 = 0;
      if (cudaDeviceGetAttribute(&pm, cudaDevAttrMaxPersistingL2CacheSize, be.device) !=
              cudaSuccess ||
          cudaDeviceGetAttribute(&wm, cudaDevAttrMaxAccessPolicyWindowSize, be.device) !=
              cudaSuccess ||
          cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, be.device) != cudaSuccess)
        pm = wm = l2 = 0;
      (void)cudaGetLastError();
      be.l2_persist_max = pm;
      be.l2_window_max = wm;
      be.l2_bytes = l2;
    }
    if (be.l2_persist_max <= 0 || be.l2_window_max <= 0 ||
        bytes + other_bytes <= (size_t)be.l2_bytes)
      return;
    const size_t carve = bytes < (size_t)be.l2_persist_max ? bytes : (size_t)be.l2_persist_max;
    // a set-aside holding less than half of the vectors gains less than the
    // smaller normal L2 loses (Jacobi-PCG on 192^3 diffusion, 30 % held: 234 ->
    // 252 us an iteration; 60-100 % held: 4-9 % faster)
    if (carve * 2 < bytes) return;
    int cur = -1;  // the limit belongs to the current device's context
    if (cudaGetDevice(&cur) != cudaSuccess || cur != be.device) {
      (void)cudaGetLastError();
      return;
    }
    L2SetAside &g = l2_set_aside(be.device);
    std::lock_guard<std::mutex> lock(g.mu);
    if (g.active == 0) {
      if (cudaDeviceGetLimit(&g.saved, cudaLimitPersistingL2CacheSize) != cudaSuccess) {
        (void)cudaGetLastError();
        return;
      }
      g.current = g.saved;
    }
    // the device's whole set-aside even where the window is smaller: with a
    // set-aside sized to the window (128^3 CG, 67 MB) the solve took 70.2 us an
    // iteration, with the whole set-aside 69.1 us
    const size_t aside = (size_t)be.l2_persist_max;
    if (aside > g.current) {
      if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, aside) != cudaSuccess) {
        (void)cudaGetLastError();
        return;
      }
      g.current = aside;
    }
    ++g.active;
    // the leading `carve` bytes of the range persist, all of them: a window
    // wider than the set-aside with a fractional hit ratio pins a random part
    // of every vector and leaves less L2 to the rest (measured slower)
    cudaAccessPolicyWindow w = {};
    w.base_ptr = base;
    w.num_bytes = carve < (size_t)be.l2_window_max ? carve : (size_t)be.l2_window_max;
    w.hitRatio = 1.0f;
    w.hitProp = cudaAccessPropertyPersisting;
    w.missProp = cudaAccessPropertyStreaming;
    be.l2_window = w;
    on = true;
  }
  ~L2Persist() {
    if (!on) return;
    be.l2_window = cudaAccessPolicyWindow{};
    (void)cudaStreamSynchronize(be.stream);
    L2SetAside &g = l2_set_aside(be.device);
    std::lock_guard<std::mutex> lock(g.mu);
    if (--g.active == 0) {
      (void)cudaCtxResetPersistingL2Cache();
      (void)cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, g.saved);
      g.current = g.saved;
    }
    (void)cudaGetLastError();
  }
  L2Persist(const L2Persist &) = delete;
  L2Persist &operator=(const L2Persist &) = delete;
};

// Starts a timed region of `kind` on the backend's stream; returns the pair
// index, or -1 when timing is off.
inline int timing_begin(Backend &be, int kind) {
  if (!be.timing) return -1;
  if (be.tev_used + 2 > be.tev.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t e;
      VCLGB_CUDA(cudaEventCreate(&e));
      be.tev.push_back(e);
    }
  }
  const int pair = (int)(be.tev_used / 2);
  if ((size_t)pair >= be.tev_kind.size()) be.tev_kind.resize(pair + 1);
  be.tev_kind[pair] = kind;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  VCLGB_CUDA(cudaStreamIsCapturing(be.stream, &cs));
  if (cs == cudaStreamCaptureStatusActive)
    VCLGB_CUDA(cudaEventRecordWithFlags(be.tev[be.tev_used], be.stream, cudaEventRecordExternal));
  else
    VCLGB_CUDA(cudaEventRecord(be.tev[be.tev_used], be.stream));
  be.tev_used += 2;
  return pair;
}
inline void timing_end(Backend &be, int pair) {
  if (pair < 0) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  VCLGB_CUDA(cudaStreamIsCapturing(be.stream, &cs));
  if (cs == cudaStreamCaptureStatusActive)
    VCLGB_CUDA(cudaEventRecordWithFlags(be.tev[2 * pair + 1], be.stream, cudaEventRecordExternal));
  else
    VCLGB_CUDA(cudaEventRecord(be.tev[2 * pair + 1], be.stream));
}
// Reads the durations of the recorded pairs (after the stream has finished
// them).  keep: the events stay in use (they are nodes of a graph that is
// replayed again).
inline void timing_collect(Backend &be, bool keep) {
  if (!be.timing || be.tev_used == 0) return;
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  for (size_t k = 0; k < be.tev_used / 2; ++k) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, be.tev[2 * k], be.tev[2 * k + 1]) == cudaSuccess)
      be.times[be.tev_kind[k] != 0].push_back(ms);
    else
      (void)cudaGetLastError();
  }
  if (!keep) be.tev_used = 0;
}

// grid size for grid-stride kernels: a whole number of waves on the 152 SMs
inline int waves_grid(const Backend &be, int threads, int blocks_per_sm_cap, size_t work_items,
                      int items_per_thread = 1) {
  int per_sm = be.max_threads_per_sm / threads;
  if (per_sm > blocks_per_sm_cap) per_sm = blocks_per_sm_cap;
  if (per_sm < 1) per_sm = 1;
  size_t full = (size_t)be.num_sms * per_sm;
  size_t need = (work_items + (size_t)threads * items_per_thread - 1) /
                ((size_t)threads * items_per_thread);
  if (need < 1) need = 1;
  return (int)(need < full ? need : full);
}

// Blocks of kernel K (launched with `threads` threads) that one SM holds at a
// time, from the occupancy calculator (registers, shared memory).  A kernel
// needing more than 32 registers a thread fits fewer than 8 blocks of 256
// threads, and a grid of 8 per SM would then run in two uneven waves.  The
// value is cached per kernel once known; a failed query is not cached.
template <auto K>
inline int resident_blocks(int threads) {
  static std::atomic<int> cached{0};
  int v = cached.load(std::memory_order_relaxed);
  if (v > 0) return v;
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, K, threads, 0) != cudaSuccess || b < 1) {
    (void)cudaGetLastError();
    return 8;
  }
  cached.store(b, std::memory_order_relaxed);
  return b;
}

// caps the grid of a grid-stride kernel at one full wave of K
template <auto K>
inline int one_wave(const Backend &be, int grid, int threads) {
  const long full = (long)be.num_sms * resident_blocks<K>(threads);
  return grid < full ? grid : (int)full;
}

// ---------------------------------------------------------------------------
// matrices
// ---------------------------------------------------------------------------
// Row-length histogram of a CSR matrix: rows of a bin need `lanes` threads
// (1..32) or, for lanes == 0, a block per row.  A matrix whose rows all fit
// one bin (identity: rows [0, count) in order) runs the single-bin kernel.
struct CsrBin {
  uint32_t lanes;      // 1,2,4,8,16,32 or 0 (= block per row)
  uint32_t count;      // rows in the bin
  uint32_t offset;     // unused (0)
  uint32_t identity;   // 1: the one bin covering all rows in order
};

constexpr int kMaxBins = 8;

// SELL chunks (32 positions of a slice) wider than this many slots are split
// over the warps of a block; a sort window sigma > 1 gathers the longest rows
// into a few slices, and one warp running such a slice alone would set the
// kernel's time.
constexpr uint32_t kSellWide = 128;

struct Transposed;  // adjoint.cu: A^T and its entry map
struct TriSolvePlan;  // precond.cu: level structure of one triangle for inplace_solve

// DIA: an internal format only (no ViennaCL counterpart), the refined
// solver's FP32 inner copy of a matrix whose entries lie on a few diagonals
// (stencils): values of diagonal d (column = row + off[d]) at vals[d*rows + row],
// zero where the diagonal leaves the matrix or the pattern has no entry.  No
// column indices are stored, so the inner product reads 4 bytes per slot.
constexpr vclgbFormat kFormatDia = static_cast<vclgbFormat>(100);
constexpr int kMaxDiag = 16;
struct DiaOffsets {  // kernel argument: the diagonals' column offsets, ascending
  int n;
  int off[kMaxDiag];
};

struct Matrix {
  vclgbFormat format = VCLGB_CSR;
  vclgbPrecision prec = VCLGB_FLOAT64;
  uint32_t rows = 0, cols = 0;
  uint64_t nnz = 0;
  size_t vsize() const { return prec == VCLGB_FLOAT64 ? 8 : 4; }

  // CSR (borrowed or owned)
  const uint32_t *row_ptr = nullptr;
  const uint32_t *col_idx = nullptr;
  const void *values = nullptr;
  DevBuf own_row_ptr, own_col_idx, own_values;
  // row-length analysis
  int num_bins = 0;
  CsrBin bins[kMaxBins];
  uint32_t max_row_len = 0;
  // reference row blocks (generate_row_block_information), built on demand
  DevBuf row_blocks;
  uint32_t num_row_blocks = 0;
  bool row_blocks_built = false;

  // ELL / HYB-ELL part: coords[item*rows + row], elems[...]
  uint32_t ell_width = 0;
  DevBuf ell_coords, ell_elems;

  // SELL-C-sigma
  uint32_t C = 32, sigma = 1, num_slices = 0;
  uint64_t sell_stored = 0;
  DevBuf sell_cpb, sell_start, sell_cols, sell_elems, sell_perm;
  DevBuf sell_wide;          // 32-position chunks wider than the warp limit
  uint32_t sell_nwide = 0;

  // HYB tail: reference CSR arrays + COO rows for the segmented kernel
  uint64_t tail_nnz = 0;     // real tail entries (0 if empty)
  DevBuf tail_rp, tail_ci, tail_v, tail_row;

  // COO (coordinate_matrix): interleaved (row, col) pairs, values, groups;
  // tail_nnz holds the entry count the segmented kernel runs over
  uint64_t coo_stored = 0;   // nnz rounded up to the reference's 128
  DevBuf coo_coords, coo_elems, coo_groups;

  // cached FP32 copy used by the mixed-precision solvers
  std::unique_ptr<Matrix> f32_copy;
  // cached FP32 copy of D^-1/2 A D^-1/2 and D^-1/2 (FP64) for refined CG,
  // and its DIA form when the matrix lies on at most kMaxDiag diagonals
  std::unique_ptr<Matrix> f32_scaled;
  std::unique_ptr<Matrix> f32_scaled_dia;
  bool f32_scaled_dia_tried = false;

  // DIA (kFormatDia)
  uint32_t dia_ndiag = 0;
  int32_t dia_off[kMaxDiag] = {};
  DevBuf dia_vals;
  DevBuf inv_sqrt_diag;
  // cached transpose for the adjoint solve
  std::shared_ptr<Transposed> transposed;
  // level structures of the triangular solves, by (upper, transposed)
  std::shared_ptr<TriSolvePlan> tri_plan[4];
  // the SpMV form the autotuner picked (tune.cu); when set, every product on
  // this matrix runs on it
  std::unique_ptr<Matrix> tuned;
  // diagonal (FP64 or FP32), built on demand for Jacobi
  DevBuf diag;
  bool diag_built = false;
};

struct Precond {
  int kind = 0;  // 1 jacobi / row scaling, 2 ilu0, 3 Chow-Patel ILU, 4 Chow-Patel ICC
  vclgbPrecision prec = VCLGB_FLOAT64;
  uint32_t rows = 0;
  DevBuf diag;   // jacobi: diag(A); ilu0: U diagonal
  DevBuf inv_diag;  // jacobi / row scaling: 1 / diag, formed once (the solvers multiply)
  // ILU0
  bool level_scheduling = true;
  uint64_t nnz = 0;
  DevBuf lu;                // factors in A's pattern
  const uint32_t *row_ptr = nullptr, *col_idx = nullptr;  // A's pattern (borrowed)
  struct Tri {
    uint32_t levels = 0;
    uint64_t rows = 0, nnz = 0;
    std::vector<uint32_t> h_level_ptr;
    DevBuf level_ptr, row_index, row_ptr, cols, vals;
    // where a run of small levels finds each value (precond.cu, level_run_kernel)
    DevBuf ecode, xcode;
    uint32_t run_width = 0;  // widest level a run may hold (0: no runs)
    int clusters = 0;        // CTAs of the cluster that runs wide runs (0: none)
  } L, U;
  // Chow-Patel: I - D_L^-1 L and I - D_U^-1 U (ICC: U = L^T) without their
  // diagonal entries, which the reference stores as zeros; diag = D_L,
  // diag_u = D_U (ICC: D_L); four work vectors for the apply
  std::unique_ptr<Matrix> cp_l, cp_u;
  DevBuf diag_u, work;
  uint32_t sweeps = 0, jacobi_iters = 0;
  // block ILU0: the block-diagonal part of A, whose pattern the factors borrow
  std::unique_ptr<Matrix> owned;
  uint32_t blocks = 0;
};

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
// Programmatic dependent launch: pdl_trigger lets the next kernel on the
// stream start its blocks (they occupy SM slots only as this kernel's blocks
// leave); pdl_wait blocks until the previous kernel has finished and its
// writes are visible (at once when this kernel was launched without the
// attribute).
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int LANES, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
  for (int o = LANES / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// NV rounded up to a power of two (at most 8)
template <int NV>
struct Pow2 { static constexpr int v = NV <= 1 ? 1 : NV <= 2 ? 2 : NV <= 4 ? 4 : 8; };

// Warp sums of NV values per lane with a halving butterfly: at each of the
// first log2(P) exchange steps a lane keeps half of its values and trades the
// other half with its partner, so the warp spends 5 + log2(P) - 1 additions
// per lane instead of 5 * NV.  On GB300 every FP64 add takes an issue slot of
// the narrow FP64 pipe, which the SpMV itself keeps busy.  The sum of value i
// ends in lane i * (32 / P); the order of additions is fixed (deterministic).
template <int NV, typename T>
__device__ __forceinline__ T warp_sum_multi(const T (&v)[NV], int lane) {
  constexpr int P = Pow2<NV>::v;
  T a[P];
#pragma unroll
  for (int i = 0; i < P; ++i) a[i] = i < NV ? v[i] : T(0);
#pragma unroll
  for (int h = P / 2, bit = 16; h >= 1; h >>= 1, bit >>= 1) {
    const bool upper = (lane & bit) != 0;
#pragma unroll
    for (int j = 0; j < h; ++j) {
      const T keep = upper ? a[j + h] : a[j];
      const T send = upper ? a[j] : a[j + h];
      a[j] = keep + __shfl_xor_sync(0xffffffffu, send, bit);
    }
  }
#pragma unroll
  for (int bit = 16 / P; bit > 0; bit >>= 1) a[0] += __shfl_xor_sync(0xffffffffu, a[0], bit);
  return a[0];
}

// Deterministic block reductions of NV values per thread; the result is
// valid in thread 0.  The FP64 adds are the cost that matters: the fused SpMV
// and vector kernels saturate the FP64 pipe.
//
// block_sum: warp butterflies, then warp 0 over the warp sums.  smem holds
// NV * (blockDim.x / 32) values, so the kernel keeps its L1 capacity (the
// SpMV kernels' x gathers hit in L1).
template <int NV, typename T>
__device__ __forceinline__ void block_sum(T (&v)[NV], T *smem) {
  constexpr int P = Pow2<NV>::v, SPAN = 32 / P;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const T w = warp_sum_multi<NV>(v, lane);
  __syncthreads();
  if ((lane & (SPAN - 1)) == 0 && lane / SPAN < NV) smem[(lane / SPAN) * nw + warp] = w;
  __syncthreads();
  if (warp == 0) {
    T t[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) t[i] = lane < nw ? smem[i * nw + lane] : T(0);
    const T s = warp_sum_multi<NV>(t, lane);
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = __shfl_sync(0xffffffffu, s, i * SPAN);
  }
}

// block_sum_wide: every thread parks its values in shared memory (no
// arithmetic), then warp 0 adds them: blockDim.x/32 adds per value plus one
// butterfly for the block, instead of a butterfly in every warp.  smem holds
// NV * blockDim.x values; used by the streaming vector passes, which gain
// nothing from L1.
template <int NV, typename T>
__device__ __forceinline__ void block_sum_wide(T (&v)[NV], T *smem) {
  constexpr int P = Pow2<NV>::v, SPAN = 32 / P;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nt = blockDim.x;
  __syncthreads();  // a previous reduction may still be reading smem
#pragma unroll
  for (int i = 0; i < NV; ++i) smem[i * nt + threadIdx.x] = v[i];
  __syncthreads();
  if (warp == 0) {
    T t[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      T a = T(0);
      for (int k = lane; k < nt; k += 32) a += smem[i * nt + k];
      t[i] = a;
    }
    const T s = warp_sum_multi<NV>(t, lane);
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = __shfl_sync(0xffffffffu, s, i * SPAN);
  }
}

// Grid-level two-stage reduction: every block writes NV partials, the last
// block to arrive sums all partials in a fixed order (deterministic) and
// returns true in thread 0 with the sums in out[].  counter is reset.
// WIDE selects block_sum_wide (smem of NV * blockDim.x values) over block_sum.
template <int NV, bool WIDE = false, typename T>
__device__ __forceinline__ bool grid_reduce(T (&v)[NV], T *partials, unsigned *counter, T *smem,
                                            T (&out)[NV]) {
  if constexpr (WIDE) block_sum_wide<NV>(v, smem);
  else block_sum<NV>(v, smem);
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) partials[(size_t)i * gridDim.x + blockIdx.x] = v[i];
    // one acquire-release ticket: it publishes this block's partials and, in
    // the block that takes the last ticket, orders the reads below after every
    // other block's partials (the barrier carries that to the whole block; a
    // fence in every thread waited for each thread's own outstanding vector
    // stores, on the serial tail)
    cuda::atomic_ref<unsigned, cuda::thread_scope_device> ticket(*counter);
    const unsigned t = ticket.fetch_add(1u, cuda::memory_order_acq_rel);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  // The other blocks' partials are read at L2 (ld.global.cg: no stale L1
  // line), every value's loads of a batch issued together -- one L2 round
  // trip for grids up to W blocks a thread -- then added in the fixed order
  // b = tid, tid + blockDim, ...  (volatile loads would be issued one after
  // another, a full L2 round trip each, on the kernel's serial tail).
  constexpr int W = NV >= 4 ? 2 : 8 / NV;
  T acc[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) acc[i] = T(0);
  for (unsigned b0 = threadIdx.x; b0 < gridDim.x; b0 += W * blockDim.x) {
    T q[NV][W];
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
      for (int k = 0; k < W; ++k) {
        const unsigned b = b0 + k * blockDim.x;
        q[i][k] = b < gridDim.x ? __ldcg(partials + (size_t)i * gridDim.x + b) : T(0);
      }
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
      for (int k = 0; k < W; ++k)
        if (b0 + k * blockDim.x < gridDim.x) acc[i] += q[i][k];
  }
  if constexpr (WIDE) block_sum_wide<NV>(acc, smem);
  else block_sum<NV>(acc, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) out[i] = acc[i];
    *counter = 0;
  }
  return threadIdx.x == 0;
}
#endif

// C-ABI plumbing
template <typename F>
vclgbStatus guarded(Backend *be, F &&f) {
  try {
    f();
    return VCLGB_SUCCESS;
  } catch (const Error &e) {
    if (be) be->last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc &) {
    if (be) be->last_error = "host allocation failed";
    return VCLGB_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    if (be) be->last_error = e.what();
    return VCLGB_GENERIC_FAILURE;
  } catch (...) {
    if (be) be->last_error = "unknown failure";
    return VCLGB_GENERIC_FAILURE;
  }
}

inline Backend *B(vclgbBackend h) { return reinterpret_cast<Backend *>(h); }
inline Matrix *M(vclgbMatrix h) { return reinterpret_cast<Matrix *>(h); }
inline Precond *P(vclgbPrecond h) { return reinterpret_cast<Precond *>(h); }

// the form a product on m runs on: the autotuned one when there is one
inline const Matrix &spmv_form(const Matrix &m) { return m.tuned ? *m.tuned : m; }

// implemented in the .cu files
void csr_analyse(Backend &be, Matrix &m);
void csr_validate(Backend &be, const Matrix &m);

}  // namespace vclgb
