// formats.cu -- CSR validation and row-length analysis, and the GPU conversions
// CSR -> ELL / SELL-C-sigma / HYB.  The reference performs these conversions on
// the host inside viennacl::copy (ell_matrix.hpp:123-171,
// sliced_ell_matrix.hpp:140-214, hyb_matrix.hpp:135-234); here every pass is a
// device kernel and the results are bit-identical to the reference layout.
#include <algorithm>
#include <cmath>

#include "formats.hpp"

namespace vclgb {

// ---------------------------------------------------------------------------
// device-wide exclusive scan (u32 in, u64 out), three passes
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename In>
__global__ void scan_tile_sums(const In *__restrict__ in, size_t n, uint64_t *tile_sums) {
  __shared__ uint64_t sm[kScanThreads / 32];
  size_t base = (size_t)blockIdx.x * kScanTile;
  uint64_t s = 0;
  for (int i = 0; i < kScanItems; ++i) {
    size_t k = base + (size_t)i * kScanThreads + threadIdx.x;
    if (k < n) s += in[k];
  }
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += sm[w];
    tile_sums[blockIdx.x] = t;
  }
}

// single block: exclusive scan of the tile sums in place, total at [ntiles]
__global__ void scan_tile_offsets(uint64_t *tile_sums, size_t ntiles) {
  __shared__ uint64_t sm[1024];
  uint64_t carry = 0;
  for (size_t base = 0; base < ntiles; base += blockDim.x) {
    size_t k = base + threadIdx.x;
    uint64_t v = k < ntiles ? tile_sums[k] : 0;
    sm[threadIdx.x] = v;
    __syncthreads();
    for (unsigned o = 1; o < blockDim.x; o <<= 1) {
      uint64_t t = threadIdx.x >= o ? sm[threadIdx.x - o] : 0;
      __syncthreads();
      sm[threadIdx.x] += t;
      __syncthreads();
    }
    uint64_t incl = sm[threadIdx.x];
    if (k < ntiles) tile_sums[k] = carry + incl - v;
    uint64_t tot = sm[blockDim.x - 1];
    __syncthreads();
    carry += tot;
  }
  if (threadIdx.x == 0) tile_sums[ntiles] = carry;
}

template <typename In, typename Out>
__global__ void scan_tiles(const In *__restrict__ in, size_t n, const uint64_t *tile_offsets,
                           Out *out) {
  __shared__ uint64_t sm[kScanTile];
  size_t base = (size_t)blockIdx.x * kScanTile;
  for (int i = 0; i < kScanItems; ++i) {
    size_t k = base + (size_t)i * kScanThreads + threadIdx.x;
    sm[i * kScanThreads + threadIdx.x] = k < n ? (uint64_t)in[k] : 0;
  }
  __syncthreads();
  // each thread scans kScanItems consecutive values
  uint64_t loc[kScanItems], s = 0;
  for (int i = 0; i < kScanItems; ++i) {
    loc[i] = s;
    s += sm[threadIdx.x * kScanItems + i];
  }
  __shared__ uint64_t ts[kScanThreads];
  ts[threadIdx.x] = s;
  __syncthreads();
  for (unsigned o = 1; o < kScanThreads; o <<= 1) {
    uint64_t t = threadIdx.x >= o ? ts[threadIdx.x - o] : 0;
    __syncthreads();
    ts[threadIdx.x] += t;
    __syncthreads();
  }
  uint64_t pre = ts[threadIdx.x] - s + tile_offsets[blockIdx.x];
  for (int i = 0; i < kScanItems; ++i) {
    size_t k = base + (size_t)threadIdx.x * kScanItems + i;
    if (k < n) out[k] = (Out)(pre + loc[i]);
  }
}

// out[0..n) = exclusive scan of in, out[n] = total (out must hold n+1); returns total
template <typename In, typename Out>
uint64_t exclusive_scan(Backend &be, const In *in, size_t n, Out *out) {
  size_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles == 0) ntiles = 1;
  DevBuf tiles((ntiles + 1) * sizeof(uint64_t), be.stream);
  scan_tile_sums<In><<<(unsigned)ntiles, kScanThreads, 0, be.stream>>>(in, n, tiles.as<uint64_t>());
  scan_tile_offsets<<<1, 1024, 0, be.stream>>>(tiles.as<uint64_t>(), ntiles);
  scan_tiles<In, Out><<<(unsigned)ntiles, kScanThreads, 0, be.stream>>>(in, n, tiles.as<uint64_t>(), out);
  be.launches += 3;
  VCLGB_CHECK_LAUNCH();
  uint64_t total = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&total, tiles.as<uint64_t>() + ntiles, sizeof(uint64_t),
                             cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  Out last = (Out)total;
  VCLGB_CUDA(cudaMemcpyAsync(out + n, &last, sizeof(Out), cudaMemcpyHostToDevice, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  return total;
}

uint64_t extern_scan_u32(Backend &be, const uint32_t *in, size_t n, uint32_t *out) {
  return exclusive_scan<uint32_t, uint32_t>(be, in, n, out);
}

// ---------------------------------------------------------------------------
// validation
// ---------------------------------------------------------------------------
__global__ void csr_validate_kernel(uint32_t rows, uint32_t cols, uint32_t nnz,
                                    const uint32_t *__restrict__ rp,
                                    const uint32_t *__restrict__ ci, unsigned *bad) {
  size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0 && (rp[0] != 0 || rp[rows] != nnz)) atomicOr(bad, 1u);
  for (size_t r = t; r < rows; r += stride)
    if (rp[r + 1] < rp[r]) atomicOr(bad, 2u);
  for (size_t k = t; k < nnz; k += stride)
    if (ci[k] >= cols) atomicOr(bad, 4u);
}

void csr_validate(Backend &be, const Matrix &m) {
  DevBuf flag(sizeof(unsigned), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(unsigned), be.stream));
  int g = waves_grid(be, 256, 8, std::max<size_t>(m.rows, m.nnz));
  csr_validate_kernel<<<g, 256, 0, be.stream>>>(m.rows, m.cols, (uint32_t)m.nnz, m.row_ptr,
                                                m.col_idx, flag.as<unsigned>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  unsigned h = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&h, flag.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  if (h & 1) throw Error(VCLGB_INVALID_MATRIX, "row_ptr[0] != 0 or row_ptr[rows] != nnz");
  if (h & 2) throw Error(VCLGB_INVALID_MATRIX, "row_ptr is not monotone");
  if (h & 4) throw Error(VCLGB_INVALID_MATRIX, "column index out of range");
}

// ---------------------------------------------------------------------------
// row-length analysis of a CSR matrix (stencil test, length histogram)
// ---------------------------------------------------------------------------
// bin of a row: 0..5 = 1,2,4,8,16,32 lanes per row (each lane issues up to 8
// loads per round, so bin q covers rows of up to 8 << q entries in one round),
// 6 = one block per row for rows longer than 4096
__device__ __host__ inline int lane_bin(uint32_t len) {
  if (len <= 8) return 0;
  if (len <= 16) return 1;
  if (len <= 32) return 2;
  if (len <= 64) return 3;
  if (len <= 128) return 4;
  if (len <= 4096) return 5;
  return 6;
}
constexpr int kLaneBins = 7;
constexpr uint32_t kBinLanes[kLaneBins] = {1, 2, 4, 8, 16, 32, 0};

__global__ void row_stats_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                 unsigned long long *stats /* [kLaneBins] counts, max, min */) {
  __shared__ unsigned cnt[kLaneBins];
  __shared__ unsigned mx, mn;
  if (threadIdx.x < kLaneBins) cnt[threadIdx.x] = 0;
  if (threadIdx.x == 0) { mx = 0; mn = 0xffffffffu; }
  __syncthreads();
  unsigned lmx = 0, lmn = 0xffffffffu;
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    uint32_t len = rp[r + 1] - rp[r];
    atomicAdd(&cnt[lane_bin(len)], 1u);
    lmx = max(lmx, len);
    lmn = min(lmn, len);
  }
  atomicMax(&mx, lmx);
  atomicMin(&mn, lmn);
  __syncthreads();
  if (threadIdx.x < kLaneBins) atomicAdd(&stats[threadIdx.x], (unsigned long long)cnt[threadIdx.x]);
  if (threadIdx.x == 0) {
    atomicMax(&stats[kLaneBins], (unsigned long long)mx);
    atomicMin(&stats[kLaneBins + 1], (unsigned long long)mn);
  }
}

void csr_analyse(Backend &be, Matrix &m) {
  DevBuf stats((kLaneBins + 2) * sizeof(unsigned long long), be.stream);
  unsigned long long init[kLaneBins + 2] = {0};
  init[kLaneBins + 1] = ~0ull;
  VCLGB_CUDA(cudaMemcpyAsync(stats.ptr, init, sizeof(init), cudaMemcpyHostToDevice, be.stream));
  int g = waves_grid(be, 256, 8, m.rows);
  row_stats_kernel<<<g, 256, 0, be.stream>>>(m.rows, m.row_ptr, stats.as<unsigned long long>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  unsigned long long h[kLaneBins + 2];
  VCLGB_CUDA(cudaMemcpyAsync(h, stats.ptr, sizeof(h), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  uint32_t maxlen = m.rows ? (uint32_t)h[kLaneBins] : 0;
  m.max_row_len = maxlen;
  double avg = m.rows ? (double)m.nnz / m.rows : 0.0;
  m.num_bins = 0;
  if (m.rows == 0) return;
  // near-uniform rows (stencils): one bin over all rows in order, no row list
  if (maxlen <= 4096 && (double)maxlen <= 2.0 * avg + 1.0) {
    CsrBin b;
    b.lanes = kBinLanes[lane_bin(maxlen)];
    b.count = m.rows;
    b.offset = 0;
    b.identity = 1;
    m.bins[0] = b;
    m.num_bins = 1;
    return;
  }
  // irregular rows: the row-window kernel classifies rows per window on the
  // fly; the bins only record the length histogram
  for (int q = 0; q < kLaneBins; ++q) {
    if (h[q] == 0) continue;
    CsrBin b;
    b.lanes = kBinLanes[q];
    b.count = (uint32_t)h[q];
    b.offset = 0;
    b.identity = 0;
    m.bins[m.num_bins++] = b;
  }
}

// ---------------------------------------------------------------------------
// reference CSR-adaptive row blocks (compressed_matrix.hpp:1152-1188), built
// like the reference from row_ptr on the host; only exported for inspection.
// ---------------------------------------------------------------------------
void csr_row_blocks(Backend &be, Matrix &m) {
  if (m.row_blocks_built) return;
  std::vector<uint32_t> rp(m.rows + 1);
  VCLGB_CUDA(cudaMemcpyAsync(rp.data(), m.row_ptr, rp.size() * sizeof(uint32_t),
                             cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  std::vector<uint32_t> blocks(m.rows + 1);
  size_t num = 0, count = 0;
  blocks[0] = 0;
  for (long i = 0; i < (long)m.rows; ++i) {
    count += rp[i + 1] - rp[i];
    if (count > 1024) {
      if ((size_t)i - blocks[num] > 0) {
        blocks[++num] = (uint32_t)i;
        --i;
      } else {
        blocks[++num] = (uint32_t)(i + 1);
      }
      count = 0;
    }
  }
  if (count > 0) blocks[++num] = m.rows;
  m.num_row_blocks = (uint32_t)num;
  m.row_blocks.alloc((num + 1) * sizeof(uint32_t), be.stream);
  VCLGB_CUDA(cudaMemcpyAsync(m.row_blocks.ptr, blocks.data(), (num + 1) * sizeof(uint32_t),
                             cudaMemcpyHostToDevice, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  m.row_blocks_built = true;
}

// ---------------------------------------------------------------------------
// ELL / HYB-ELL fill: thread per row writes slots j*rows + row (coalesced in j)
// ---------------------------------------------------------------------------
template <typename W>
__global__ void ell_fill_kernel(uint32_t rows, uint32_t width, const uint32_t *__restrict__ rp,
                                const uint32_t *__restrict__ ci, const W *__restrict__ v,
                                uint32_t *coords, W *elems) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    uint32_t s = rp[r], e = rp[r + 1];
    uint32_t len = e - s < width ? e - s : width;
    for (uint32_t j = 0; j < len; ++j) {
      size_t off = (size_t)j * rows + r;
      coords[off] = ci[s + j];
      elems[off] = v[s + j];
    }
  }
}

template <typename W>
static void ell_fill(Backend &be, const Matrix &src, uint32_t width, Matrix &dst) {
  size_t slots = (size_t)src.rows * width;
  dst.ell_coords.alloc(std::max<size_t>(slots, 1) * sizeof(uint32_t), be.stream);
  dst.ell_elems.alloc(std::max<size_t>(slots, 1) * sizeof(W), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(dst.ell_coords.ptr, 0, dst.ell_coords.bytes, be.stream));
  VCLGB_CUDA(cudaMemsetAsync(dst.ell_elems.ptr, 0, dst.ell_elems.bytes, be.stream));
  if (slots) {
    int g = waves_grid(be, 256, 8, src.rows);
    ell_fill_kernel<W><<<g, 256, 0, be.stream>>>(src.rows, width, src.row_ptr, src.col_idx,
                                                 static_cast<const W *>(src.values),
                                                 dst.ell_coords.as<uint32_t>(),
                                                 dst.ell_elems.as<W>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  }
}

static void copy_header(const Matrix &src, Matrix &dst, vclgbFormat f) {
  dst.format = f;
  dst.prec = src.prec;
  dst.rows = src.rows;
  dst.cols = src.cols;
  dst.nnz = src.nnz;
}

std::unique_ptr<Matrix> convert_ell(Backend &be, const Matrix &csr) {
  require(csr.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "conversion source must be CSR");
  auto out = std::make_unique<Matrix>();
  copy_header(csr, *out, VCLGB_ELL);
  out->ell_width = csr.max_row_len;
  if (csr.prec == VCLGB_FLOAT64)
    ell_fill<uint64_t>(be, csr, out->ell_width, *out);
  else
    ell_fill<uint32_t>(be, csr, out->ell_width, *out);
  return out;
}

// ---------------------------------------------------------------------------
// SELL-C-sigma
// ---------------------------------------------------------------------------
// one block per window of sigma rows: rank = stable position in decreasing length
__global__ void sell_sort_kernel(uint32_t rows, uint32_t sigma, const uint32_t *__restrict__ rp,
                                 uint32_t *perm) {
  extern __shared__ uint32_t lens[];
  size_t w0 = (size_t)blockIdx.x * sigma;
  uint32_t wn = (uint32_t)min((size_t)sigma, (size_t)rows - w0);
  for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) lens[i] = rp[w0 + i + 1] - rp[w0 + i];
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < wn; i += blockDim.x) {
    uint32_t li = lens[i], rank = 0;
    for (uint32_t j = 0; j < wn; ++j) {
      uint32_t lj = lens[j];
      rank += (lj > li) || (lj == li && j < i);
    }
    perm[w0 + rank] = (uint32_t)(w0 + i);
  }
}

__global__ void sell_width_kernel(uint32_t rows, uint32_t C, uint32_t nslices,
                                  const uint32_t *__restrict__ rp,
                                  const uint32_t *__restrict__ perm, uint32_t *cpb,
                                  uint32_t *slots /* cpb*C, for the scan */) {
  for (size_t s = (size_t)blockIdx.x * blockDim.x + threadIdx.x; s < nslices;
       s += (size_t)gridDim.x * blockDim.x) {
    uint32_t w = 0;
    for (uint32_t l = 0; l < C; ++l) {
      size_t pos = s * C + l;
      if (pos >= rows) break;
      uint32_t r = perm ? perm[pos] : (uint32_t)pos;
      w = max(w, rp[r + 1] - rp[r]);
    }
    cpb[s] = w;
    slots[s] = w * C;
  }
}

template <typename W>
__global__ void sell_fill_kernel(uint32_t rows, uint32_t C, const uint32_t *__restrict__ rp,
                                 const uint32_t *__restrict__ ci, const W *__restrict__ v,
                                 const uint32_t *__restrict__ perm,
                                 const uint32_t *__restrict__ start, uint32_t *cols, W *elems) {
  for (size_t pos = (size_t)blockIdx.x * blockDim.x + threadIdx.x; pos < rows;
       pos += (size_t)gridDim.x * blockDim.x) {
    uint32_t s = (uint32_t)(pos / C), l = (uint32_t)(pos % C);
    uint32_t r = perm ? perm[pos] : (uint32_t)pos;
    uint32_t b = rp[r], e = rp[r + 1];
    size_t base = (size_t)start[s] + l;
    for (uint32_t j = 0; b + j < e; ++j) {
      cols[base + (size_t)j * C] = ci[b + j];
      elems[base + (size_t)j * C] = v[b + j];
    }
  }
}

std::unique_ptr<Matrix> convert_sell(Backend &be, const Matrix &csr, uint32_t C, uint32_t sigma) {
  require(csr.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "conversion source must be CSR");
  if (C == 0) C = 32;  // sliced_ell_matrix.hpp:146-147 default
  if (sigma == 0) sigma = 1;
  require(sigma <= 8192, VCLGB_INVALID_ARGUMENT, "sigma must be <= 8192");
  auto out = std::make_unique<Matrix>();
  copy_header(csr, *out, VCLGB_SELL);
  out->C = C;
  out->sigma = sigma;
  uint32_t rows = csr.rows;
  if (rows == 0) return out;
  uint32_t nslices = (rows - 1) / C + 1;
  out->num_slices = nslices;
  const uint32_t *perm = nullptr;
  if (sigma > 1) {
    out->sell_perm.alloc((size_t)rows * sizeof(uint32_t), be.stream);
    uint32_t nwin = (rows + sigma - 1) / sigma;
    sell_sort_kernel<<<nwin, 256, sigma * sizeof(uint32_t), be.stream>>>(
        rows, sigma, csr.row_ptr, out->sell_perm.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    perm = out->sell_perm.as<uint32_t>();
  }
  out->sell_cpb.alloc((size_t)nslices * sizeof(uint32_t), be.stream);
  out->sell_start.alloc(((size_t)nslices + 1) * sizeof(uint32_t), be.stream);
  DevBuf slots((size_t)nslices * sizeof(uint32_t), be.stream);
  int g = waves_grid(be, 256, 8, nslices);
  sell_width_kernel<<<g, 256, 0, be.stream>>>(rows, C, nslices, csr.row_ptr, perm,
                                              out->sell_cpb.as<uint32_t>(), slots.as<uint32_t>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  DevBuf start64(((size_t)nslices + 1) * sizeof(uint64_t), be.stream);
  uint64_t total = exclusive_scan<uint32_t, uint64_t>(be, slots.as<uint32_t>(), nslices,
                                                      start64.as<uint64_t>());
  require(total < (1ull << 32), VCLGB_INVALID_ARGUMENT,
          "SELL storage exceeds the 32-bit block_start of sliced_ell_matrix");
  // narrow to u32 block_start (the reference IndexT)
  exclusive_scan<uint32_t, uint32_t>(be, slots.as<uint32_t>(), nslices,
                                     out->sell_start.as<uint32_t>());
  out->sell_stored = total;
  size_t vs = csr.vsize();
  out->sell_cols.alloc(std::max<uint64_t>(total, 1) * sizeof(uint32_t), be.stream);
  out->sell_elems.alloc(std::max<uint64_t>(total, 1) * vs, be.stream);
  VCLGB_CUDA(cudaMemsetAsync(out->sell_cols.ptr, 0, out->sell_cols.bytes, be.stream));
  VCLGB_CUDA(cudaMemsetAsync(out->sell_elems.ptr, 0, out->sell_elems.bytes, be.stream));
  int g2 = waves_grid(be, 256, 8, rows);
  if (vs == 8)
    sell_fill_kernel<uint64_t><<<g2, 256, 0, be.stream>>>(
        rows, C, csr.row_ptr, csr.col_idx, static_cast<const uint64_t *>(csr.values), perm,
        out->sell_start.as<uint32_t>(), out->sell_cols.as<uint32_t>(),
        out->sell_elems.as<uint64_t>());
  else
    sell_fill_kernel<uint32_t><<<g2, 256, 0, be.stream>>>(
        rows, C, csr.row_ptr, csr.col_idx, static_cast<const uint32_t *>(csr.values), perm,
        out->sell_start.as<uint32_t>(), out->sell_cols.as<uint32_t>(),
        out->sell_elems.as<uint32_t>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  sell_wide_chunks(be, *out);
  return out;
}

// List of the 32-position chunks wider than kSellWide slots (C a multiple of
// 32), which the SELL kernel hands to whole blocks.
void sell_wide_chunks(Backend &be, Matrix &m) {
  m.sell_wide.release();
  m.sell_nwide = 0;
  if (m.rows == 0 || m.C % 32 != 0) return;
  std::vector<uint32_t> cpb(m.num_slices);
  VCLGB_CUDA(cudaMemcpyAsync(cpb.data(), m.sell_cpb.ptr, (size_t)m.num_slices * 4,
                             cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  const uint32_t per = m.C / 32, nsub = (m.rows + 31) / 32;
  std::vector<uint32_t> wide;
  for (uint32_t s = 0; s < m.num_slices; ++s) {
    if (cpb[s] <= kSellWide) continue;
    for (uint32_t k = 0; k < per && s * per + k < nsub; ++k) wide.push_back(s * per + k);
  }
  if (wide.empty()) return;
  m.sell_wide.alloc(wide.size() * 4, be.stream);
  VCLGB_CUDA(cudaMemcpyAsync(m.sell_wide.ptr, wide.data(), wide.size() * 4,
                             cudaMemcpyHostToDevice, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  m.sell_nwide = (uint32_t)wide.size();
}

// ---------------------------------------------------------------------------
// HYB
// ---------------------------------------------------------------------------
__global__ void len_hist_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                unsigned long long *hist) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x)
    atomicAdd(&hist[rp[r + 1] - rp[r]], 1ull);
}

__global__ void tail_len_kernel(uint32_t rows, uint32_t width, const uint32_t *__restrict__ rp,
                                uint32_t *tlen) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    uint32_t len = rp[r + 1] - rp[r];
    tlen[r] = len > width ? len - width : 0;
  }
}

template <typename W>
__global__ void tail_fill_kernel(uint32_t rows, uint32_t width, const uint32_t *__restrict__ rp,
                                 const uint32_t *__restrict__ ci, const W *__restrict__ v,
                                 const uint32_t *__restrict__ trp, uint32_t *tci, W *tv,
                                 uint32_t *trow) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    uint32_t s = rp[r] + width, e = rp[r + 1];
    uint32_t o = trp[r];
    for (uint32_t k = s; k < e; ++k, ++o) {
      tci[o] = ci[k];
      tv[o] = v[k];
      trow[o] = (uint32_t)r;
    }
  }
}

std::unique_ptr<Matrix> convert_hyb(Backend &be, const Matrix &csr, double threshold) {
  require(csr.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "conversion source must be CSR");
  auto out = std::make_unique<Matrix>();
  copy_header(csr, *out, VCLGB_HYB);
  uint32_t rows = csr.rows, maxlen = csr.max_row_len;
  // width rule of hyb_matrix.hpp:146-163, evaluated in the value precision
  uint32_t width = maxlen;
  if (rows > 0) {
    DevBuf hist(((size_t)maxlen + 1) * sizeof(unsigned long long), be.stream);
    VCLGB_CUDA(cudaMemsetAsync(hist.ptr, 0, hist.bytes, be.stream));
    int g = waves_grid(be, 256, 8, rows);
    len_hist_kernel<<<g, 256, 0, be.stream>>>(rows, csr.row_ptr, hist.as<unsigned long long>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    std::vector<unsigned long long> h(maxlen + 1);
    VCLGB_CUDA(cudaMemcpyAsync(h.data(), hist.ptr, hist.bytes, cudaMemcpyDeviceToHost, be.stream));
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    unsigned long long sum = 0;
    for (uint32_t ind = 0; ind <= maxlen; ++ind) {
      sum += h[ind];
      bool hit = csr.prec == VCLGB_FLOAT32
                     ? (float)sum >= (float)threshold * (float)rows
                     : (double)sum >= threshold * (double)rows;
      if (hit) { width = ind; break; }
    }
  }
  out->ell_width = width;
  if (csr.prec == VCLGB_FLOAT64)
    ell_fill<uint64_t>(be, csr, width, *out);
  else
    ell_fill<uint32_t>(be, csr, width, *out);
  // tail: row_ptr by scan of the per-row overflow, then entries + COO rows
  out->tail_rp.alloc(((size_t)rows + 1) * sizeof(uint32_t), be.stream);
  DevBuf tlen(std::max<size_t>(rows, 1) * sizeof(uint32_t), be.stream);
  uint64_t tnnz = 0;
  if (rows > 0) {
    int g = waves_grid(be, 256, 8, rows);
    tail_len_kernel<<<g, 256, 0, be.stream>>>(rows, width, csr.row_ptr, tlen.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    tnnz = exclusive_scan<uint32_t, uint32_t>(be, tlen.as<uint32_t>(), rows,
                                              out->tail_rp.as<uint32_t>());
  } else {
    VCLGB_CUDA(cudaMemsetAsync(out->tail_rp.ptr, 0, sizeof(uint32_t), be.stream));
  }
  out->tail_nnz = tnnz;
  size_t vs = csr.vsize();
  size_t cap = std::max<uint64_t>(tnnz, 1);  // empty tail: one placeholder entry (hyb_matrix.hpp:213-217)
  out->tail_ci.alloc(cap * sizeof(uint32_t), be.stream);
  out->tail_v.alloc(cap * vs, be.stream);
  out->tail_row.alloc(cap * sizeof(uint32_t), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(out->tail_ci.ptr, 0, out->tail_ci.bytes, be.stream));
  VCLGB_CUDA(cudaMemsetAsync(out->tail_v.ptr, 0, out->tail_v.bytes, be.stream));
  if (tnnz > 0) {
    int g = waves_grid(be, 256, 8, rows);
    if (vs == 8)
      tail_fill_kernel<uint64_t><<<g, 256, 0, be.stream>>>(
          rows, width, csr.row_ptr, csr.col_idx, static_cast<const uint64_t *>(csr.values),
          out->tail_rp.as<uint32_t>(), out->tail_ci.as<uint32_t>(), out->tail_v.as<uint64_t>(),
          out->tail_row.as<uint32_t>());
    else
      tail_fill_kernel<uint32_t><<<g, 256, 0, be.stream>>>(
          rows, width, csr.row_ptr, csr.col_idx, static_cast<const uint32_t *>(csr.values),
          out->tail_rp.as<uint32_t>(), out->tail_ci.as<uint32_t>(), out->tail_v.as<uint32_t>(),
          out->tail_row.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  }
  return out;
}

// ---------------------------------------------------------------------------
// COO (coordinate_matrix.hpp:46-101): (row, col) pairs interleaved, values,
// both zero-padded to a multiple of 128 entries (AlignmentV = 128), and the
// 65 group boundaries of the reference's copy().
// ---------------------------------------------------------------------------
constexpr uint64_t kCooAlign = 128;

template <typename V>
__global__ void coo_fill_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                const uint32_t *__restrict__ ci, const V *__restrict__ vals,
                                uint2 *coords, V *elems) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x)
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k) {
      coords[k] = make_uint2((uint32_t)r, ci[k]);
      elems[k] = vals[k];
    }
}

// The reference's boundary loop (coordinate_matrix.hpp:74-91) compares the
// running entry count with vcl_size_t((f+1)/64.0) * nnz: the cast truncates
// the ratio, so the bound is 0 for every f < 63.  Group 0 therefore ends
// after the first non-empty row, groups 1..62 are empty and group 63 holds
// the rest; this kernel writes exactly that (d1 = entries of the first row).
__global__ void coo_groups_kernel(uint64_t nnz, const uint2 *__restrict__ coords,
                                  uint32_t *groups) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint64_t d1 = 0;
  if (nnz > 0) {
    const uint32_t row0 = coords[0].x;
    uint64_t lo = 1, hi = nnz;  // first k with coords[k].x != row0 (rows sorted)
    while (lo < hi) {
      const uint64_t mid = lo + (hi - lo) / 2;
      if (coords[mid].x == row0) lo = mid + 1;
      else hi = mid;
    }
    d1 = lo;
  }
  groups[0] = 0;
  for (int g = 1; g < 64; ++g) groups[g] = (uint32_t)d1;
  groups[64] = (uint32_t)nnz;
}

void coo_groups(Backend &be, Matrix &m) {
  m.coo_groups.alloc(65 * sizeof(uint32_t), be.stream);
  coo_groups_kernel<<<1, 32, 0, be.stream>>>(m.tail_nnz, m.coo_coords.as<uint2>(),
                                             m.coo_groups.as<uint32_t>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
}

std::unique_ptr<Matrix> convert_coo(Backend &be, const Matrix &csr) {
  require(csr.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "conversion source must be CSR");
  auto out = std::make_unique<Matrix>();
  copy_header(csr, *out, VCLGB_COO);
  const uint64_t nnz = csr.nnz;
  const uint64_t stored = (nnz + kCooAlign - 1) / kCooAlign * kCooAlign;
  const size_t vs = csr.vsize();
  out->coo_stored = stored;
  out->tail_nnz = nnz;
  out->coo_coords.alloc(std::max<uint64_t>(stored, 1) * 2 * sizeof(uint32_t), be.stream);
  out->coo_elems.alloc(std::max<uint64_t>(stored, 1) * vs, be.stream);
  VCLGB_CUDA(cudaMemsetAsync(out->coo_coords.ptr, 0, out->coo_coords.bytes, be.stream));
  VCLGB_CUDA(cudaMemsetAsync(out->coo_elems.ptr, 0, out->coo_elems.bytes, be.stream));
  if (nnz > 0) {
    int g = waves_grid(be, 256, 8, csr.rows);
    if (vs == 8)
      coo_fill_kernel<uint64_t><<<g, 256, 0, be.stream>>>(
          csr.rows, csr.row_ptr, csr.col_idx, static_cast<const uint64_t *>(csr.values),
          out->coo_coords.as<uint2>(), out->coo_elems.as<uint64_t>());
    else
      coo_fill_kernel<uint32_t><<<g, 256, 0, be.stream>>>(
          csr.rows, csr.row_ptr, csr.col_idx, static_cast<const uint32_t *>(csr.values),
          out->coo_coords.as<uint2>(), out->coo_elems.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  }
  coo_groups(be, *out);
  return out;
}

// wrapped COO arrays: rows sorted and in range, columns in range
__global__ void coo_validate_kernel(uint64_t nnz, uint32_t rows, uint32_t cols,
                                    const uint2 *__restrict__ coords, unsigned *bad) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (size_t)gridDim.x * blockDim.x) {
    const uint2 rc = coords[k];
    if (rc.x >= rows) atomicOr(bad, 1u);
    if (rc.y >= cols) atomicOr(bad, 2u);
    if (k > 0 && coords[k - 1].x > rc.x) atomicOr(bad, 4u);
  }
}

void coo_validate(Backend &be, const Matrix &m) {
  if (m.tail_nnz == 0) return;
  DevBuf flag(sizeof(unsigned), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(unsigned), be.stream));
  int g = waves_grid(be, 256, 8, m.tail_nnz);
  coo_validate_kernel<<<g, 256, 0, be.stream>>>(m.tail_nnz, m.rows, m.cols,
                                                m.coo_coords.as<uint2>(), flag.as<unsigned>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  unsigned h = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&h, flag.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  if (h & 1) throw Error(VCLGB_INVALID_MATRIX, "COO row index out of range");
  if (h & 2) throw Error(VCLGB_INVALID_MATRIX, "COO column index out of range");
  if (h & 4) throw Error(VCLGB_INVALID_MATRIX, "COO entries are not sorted by row");
}

// ---------------------------------------------------------------------------
// DIA (internal): diagonal offsets by a hash set in global memory, then the
// values by diagonal
// ---------------------------------------------------------------------------
constexpr int kDiaSlots = 64;
constexpr int kDiaEmpty = INT32_MIN;

__global__ void dia_offsets_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                   const uint32_t *__restrict__ ci, int *table, unsigned *count,
                                   unsigned *overflow) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    if (*(volatile unsigned *)overflow) return;
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k) {
      const int64_t d = (int64_t)ci[k] - (int64_t)r;
      if (d <= INT32_MIN || d > INT32_MAX) {
        atomicOr(overflow, 1u);
        return;
      }
      const int off = (int)d;
      unsigned h = ((unsigned)off * 2654435761u) >> 26;  // 64 slots
      for (int probe = 0; probe < kDiaSlots; ++probe, h = (h + 1) & (kDiaSlots - 1)) {
        const int seen = *(volatile int *)(table + h);
        if (seen == off) break;
        if (seen == kDiaEmpty) {
          const int prev = atomicCAS(table + h, kDiaEmpty, off);
          if (prev == kDiaEmpty) {
            if (atomicAdd(count, 1u) >= (unsigned)kMaxDiag) atomicOr(overflow, 1u);
            break;
          }
          if (prev == off) break;
        }
      }
    }
  }
}

template <typename V>
__global__ void dia_fill_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                const uint32_t *__restrict__ ci, const V *__restrict__ v,
                                DiaOffsets offs, V *vals) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k) {
      const int off = (int)((int64_t)ci[k] - (int64_t)r);
      int d = 0;
      while (d < offs.n && offs.off[d] != off) ++d;
      if (d < offs.n) vals[(size_t)d * rows + r] += v[k];  // repeated entries add up
    }
  }
}

std::unique_ptr<Matrix> try_convert_dia(Backend &be, const Matrix &csr, double max_fill) {
  require(csr.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "conversion source must be CSR");
  if (csr.rows == 0 || csr.nnz == 0) return nullptr;
  if (csr.rows >= (1u << 31) || csr.cols >= (1u << 31)) return nullptr;  // 32-bit indexing
  DevBuf table(kDiaSlots * sizeof(int), be.stream), flags(2 * sizeof(unsigned), be.stream);
  std::vector<int> h(kDiaSlots, kDiaEmpty);
  VCLGB_CUDA(cudaMemcpyAsync(table.ptr, h.data(), kDiaSlots * sizeof(int),
                             cudaMemcpyHostToDevice, be.stream));
  VCLGB_CUDA(cudaMemsetAsync(flags.ptr, 0, flags.bytes, be.stream));
  int g = waves_grid(be, 256, 8, csr.rows);
  dia_offsets_kernel<<<g, 256, 0, be.stream>>>(csr.rows, csr.row_ptr, csr.col_idx,
                                               table.as<int>(), flags.as<unsigned>(),
                                               flags.as<unsigned>() + 1);
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  unsigned hf[2] = {0, 0};
  VCLGB_CUDA(cudaMemcpyAsync(h.data(), table.ptr, kDiaSlots * sizeof(int),
                             cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaMemcpyAsync(hf, flags.ptr, sizeof(hf), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  if (hf[1] || hf[0] > (unsigned)kMaxDiag) return nullptr;
  std::vector<int> offs;
  for (int x : h)
    if (x != kDiaEmpty) offs.push_back(x);
  std::sort(offs.begin(), offs.end());
  const double stored = (double)offs.size() * csr.rows;
  if (stored > max_fill * (double)csr.nnz || stored >= 4294967296.0) return nullptr;
  auto out = std::make_unique<Matrix>();
  copy_header(csr, *out, kFormatDia);
  out->dia_ndiag = (uint32_t)offs.size();
  DiaOffsets o;
  o.n = (int)offs.size();
  for (int d = 0; d < kMaxDiag; ++d) {
    o.off[d] = d < o.n ? offs[d] : 0;
    out->dia_off[d] = o.off[d];
  }
  const size_t vs = csr.vsize();
  out->dia_vals.alloc((size_t)o.n * csr.rows * vs, be.stream);
  VCLGB_CUDA(cudaMemsetAsync(out->dia_vals.ptr, 0, out->dia_vals.bytes, be.stream));
  if (vs == 8)
    dia_fill_kernel<double><<<g, 256, 0, be.stream>>>(csr.rows, csr.row_ptr, csr.col_idx,
                                                      static_cast<const double *>(csr.values), o,
                                                      out->dia_vals.as<double>());
  else
    dia_fill_kernel<float><<<g, 256, 0, be.stream>>>(csr.rows, csr.row_ptr, csr.col_idx,
                                                     static_cast<const float *>(csr.values), o,
                                                     out->dia_vals.as<float>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  return out;
}

__global__ void tail_rows_kernel(uint32_t rows, const uint32_t *__restrict__ trp, uint32_t *trow) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x)
    for (uint32_t k = trp[r]; k < trp[r + 1]; ++k) trow[k] = (uint32_t)r;
}

void tail_rows_from_rp(Backend &be, uint32_t rows, const uint32_t *trp, uint64_t tnnz,
                       uint32_t *trow) {
  if (!rows || !tnnz) return;
  int g = waves_grid(be, 256, 8, rows);
  tail_rows_kernel<<<g, 256, 0, be.stream>>>(rows, trp, trow);
  be.launches++;
  VCLGB_CHECK_LAUNCH();
}

// ---------------------------------------------------------------------------
// FP32 copy (same format, same index arrays shared by value copy)
// ---------------------------------------------------------------------------
__global__ void d2f_kernel(size_t n, const double *__restrict__ in, float *out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = (float)in[i];
}

static void d2f(Backend &be, size_t n, const void *in, DevBuf &out) {
  out.alloc(std::max<size_t>(n, 1) * sizeof(float), be.stream);
  if (!n) return;
  int g = waves_grid(be, 256, 8, n);
  d2f_kernel<<<g, 256, 0, be.stream>>>(n, static_cast<const double *>(in), out.as<float>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
}

std::unique_ptr<Matrix> convert_f32(Backend &be, const Matrix &m) {
  require(m.prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "matrix is already FP32");
  auto out = std::make_unique<Matrix>();
  copy_header(m, *out, m.format);
  out->prec = VCLGB_FLOAT32;
  switch (m.format) {
    case VCLGB_CSR:
      out->row_ptr = m.row_ptr;
      out->col_idx = m.col_idx;
      d2f(be, m.nnz, m.values, out->own_values);
      out->values = out->own_values.ptr;
      out->num_bins = m.num_bins;
      for (int i = 0; i < m.num_bins; ++i) out->bins[i] = m.bins[i];
      out->max_row_len = m.max_row_len;
      break;
    default:
      throw Error(VCLGB_UNSUPPORTED, "FP32 copies are built from CSR matrices");
  }
  return out;
}

}  // namespace vclgb
