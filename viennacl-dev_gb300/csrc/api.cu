// api.cu -- the extern "C" entry points declared in include/vclgb.h.
#include <algorithm>

#include <cstdlib>

#include "formats.hpp"
#include "vecpass.cuh"

namespace vclgb {
template <typename T>
void cg_solve(Backend &, Matrix &, const T *, T *, vclgbSolverTag *, const Precond *);
template <typename T>
void bicgstab_solve(Backend &, Matrix &, const T *, T *, vclgbSolverTag *, const Precond *);
template <typename T>
void gmres_solve(Backend &, Matrix &, const T *, T *, vclgbSolverTag *, const Precond *);
void mixed_cg_solve(Backend &, Matrix &, const double *, double *, vclgbSolverTag *, float);
void refined_cg_solve(Backend &, Matrix &, const double *, double *, vclgbSolverTag *, double,
                      uint32_t, uint32_t *);
struct Batch;
Batch *batch_create(Backend &, const Matrix &, uint32_t, const uint32_t *, const int32_t *);
void batch_tune(Backend &, Batch &, const double *);
bool batch_solve(Backend &, Batch &, const double *, double *, double, uint32_t, uint32_t *,
                 int32_t *, double *);
void batch_config(const Batch &, int *, int *);
void batch_destroy(Batch *);
template <typename T>
void adjoint_solve(Backend &, Matrix &, int, const Precond *, const T *, const T *, T *, T *,
                   vclgbSolverTag *, bool);
void transpose_export(Backend &, Matrix &, int, void *);
}  // namespace vclgb

using namespace vclgb;

namespace {
template <class F>
static vclgbStatus convert(vclgbBackend h, vclgbMatrix src, vclgbMatrix *out, F &&f) {
  if (!h || !src || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    std::unique_ptr<Matrix> m = f(*be, *M(src));
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbMatrix>(m.release());
  });
}

template <class F>
static vclgbStatus solve_entry(vclgbBackend h, vclgbMatrix A, const void *b, void *x,
                               vclgbSolverTag *tag, F &&f) {
  if (!h || !A || !tag || !b || !x) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  vclgbStatus s = guarded(be, [&]() { f(*be, *M(A)); });
  if (s != VCLGB_SUCCESS) {
    tag->status = s;
    return s;
  }
  return (vclgbStatus)tag->status;
}

}  // namespace

extern "C" {

VCLGB_API const char *vclgbVersion(void) { return "vclgb 0.1 (sm_103a)"; }

VCLGB_API vclgbStatus vclgbBackendCreate(vclgbBackend *out, void *stream) {
  if (!out) return VCLGB_INVALID_ARGUMENT;
  auto be = new (std::nothrow) Backend();
  if (!be) return VCLGB_OUT_OF_MEMORY;
  vclgbStatus s = guarded(be, [&]() {
    VCLGB_CUDA(cudaGetDevice(&be->device));
    cudaDeviceProp prop;
    VCLGB_CUDA(cudaGetDeviceProperties(&prop, be->device));
    be->num_sms = prop.multiProcessorCount;
    be->max_threads_per_sm = prop.maxThreadsPerMultiProcessor;
    be->max_smem_per_block = prop.sharedMemPerBlockOptin;
    if (const char *e = std::getenv("VCLGB_PDL")) be->pdl = std::strcmp(e, "1") == 0;
    if (stream) {
      be->stream = static_cast<cudaStream_t>(stream);
    } else {
      // a blocking stream of our own: ordered with the legacy default stream,
      // and capturable into CUDA graphs
      VCLGB_CUDA(cudaStreamCreateWithFlags(&be->stream, cudaStreamDefault));
      be->own_stream = true;
    }
    VCLGB_CUDA(cudaMallocHost(&be->host_flags, 64));
    be->red_partials.alloc(8 * kMaxSpmvGrid * sizeof(double), be->stream);
    be->red_counter.alloc(64, be->stream);
    VCLGB_CUDA(cudaMemsetAsync(be->red_counter.ptr, 0, 64, be->stream));
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
  });
  if (s != VCLGB_SUCCESS) {
    delete be;
    return s;
  }
  *out = reinterpret_cast<vclgbBackend>(be);
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbBackendDestroy(vclgbBackend *h) {
  if (!h || !*h) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(*h);
  cudaStreamSynchronize(be->stream);
  be->release_buffers();
  cudaStreamSynchronize(be->stream);
  if (be->host_flags) cudaFreeHost(be->host_flags);
  for (cudaEvent_t e : be->tev) cudaEventDestroy(e);
  for (cudaEvent_t e : be->poll_ev)
    if (e) cudaEventDestroy(e);
  if (be->own_stream) cudaStreamDestroy(be->stream);
  if (be->retired_stream) cudaStreamDestroy(be->retired_stream);
  delete be;
  *h = nullptr;
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbBackendSetStream(vclgbBackend h, void *stream) {
  if (!h) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(stream != nullptr, VCLGB_INVALID_ARGUMENT, "stream must not be NULL");
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    if (be->own_stream) {
      // matrices and preconditioners made on it still free their scratch on it
      if (be->retired_stream) VCLGB_CUDA(cudaStreamDestroy(be->retired_stream));
      be->retired_stream = be->stream;
    }
    be->own_stream = false;
    be->stream = static_cast<cudaStream_t>(stream);
    be->adopt_stream(be->stream);
  });
}

VCLGB_API vclgbStatus vclgbBackendSynchronize(vclgbBackend h) {
  if (!h) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { VCLGB_CUDA(cudaStreamSynchronize(be->stream)); });
}

VCLGB_API const char *vclgbBackendLastError(vclgbBackend h) {
  return h ? B(h)->last_error.c_str() : "no backend";
}

VCLGB_API uint64_t vclgbBackendLaunchCount(vclgbBackend h) { return h ? B(h)->launches : 0; }

VCLGB_API vclgbStatus vclgbBackendSetKernelTiming(vclgbBackend h, int enable) {
  if (!h) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    timing_collect(*be, false);
    be->timing = enable != 0;
    if (be->timing && be->tev.size() < 1024) {
      while (be->tev.size() < 1024) {
        cudaEvent_t e;
        VCLGB_CUDA(cudaEventCreate(&e));
        be->tev.push_back(e);
      }
    }
    be->times[0].clear();
    be->times[1].clear();
  });
}

VCLGB_API vclgbStatus vclgbBackendKernelTimes(vclgbBackend h, int kind, float *out,
                                              uint64_t capacity, uint64_t *count) {
  if (!h || !count || (kind != 0 && kind != 1)) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    timing_collect(*be, false);
    std::vector<float> &t = be->times[kind];
    *count = t.size();
    if (out) std::memcpy(out, t.data(), std::min<uint64_t>(capacity, t.size()) * sizeof(float));
    t.clear();
  });
}

// ---------------------------------------------------------------------------
VCLGB_API vclgbStatus vclgbCsrCreate(vclgbBackend h, vclgbPrecision prec, uint32_t rows,
                                     uint32_t cols, uint32_t nnz, const uint32_t *d_row_ptr,
                                     const uint32_t *d_col_idx, const void *d_values,
                                     vclgbMatrix *out) {
  if (!h || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(prec == VCLGB_FLOAT32 || prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "bad precision");
    require(d_row_ptr != nullptr, VCLGB_INVALID_ARGUMENT, "row_ptr is NULL");
    require(nnz == 0 || (d_col_idx && d_values), VCLGB_INVALID_ARGUMENT, "cols/values are NULL");
    auto m = std::make_unique<Matrix>();
    m->format = VCLGB_CSR;
    m->prec = prec;
    m->rows = rows;
    m->cols = cols;
    m->nnz = nnz;
    m->row_ptr = d_row_ptr;
    m->col_idx = d_col_idx;
    m->values = d_values;
    csr_validate(*be, *m);
    csr_analyse(*be, *m);
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbMatrix>(m.release());
  });
}

VCLGB_API vclgbStatus vclgbMatrixToEll(vclgbBackend h, vclgbMatrix csr, vclgbMatrix *out) {
  return convert(h, csr, out, [](Backend &be, Matrix &m) { return convert_ell(be, m); });
}
VCLGB_API vclgbStatus vclgbMatrixToSell(vclgbBackend h, vclgbMatrix csr, uint32_t C,
                                        uint32_t sigma, vclgbMatrix *out) {
  return convert(h, csr, out,
                 [&](Backend &be, Matrix &m) { return convert_sell(be, m, C, sigma); });
}
VCLGB_API vclgbStatus vclgbMatrixToHyb(vclgbBackend h, vclgbMatrix csr, double thr,
                                       vclgbMatrix *out) {
  return convert(h, csr, out, [&](Backend &be, Matrix &m) { return convert_hyb(be, m, thr); });
}
VCLGB_API vclgbStatus vclgbMatrixToCoo(vclgbBackend h, vclgbMatrix csr, vclgbMatrix *out) {
  return convert(h, csr, out, [](Backend &be, Matrix &m) { return convert_coo(be, m); });
}
VCLGB_API vclgbStatus vclgbMatrixToFloat32(vclgbBackend h, vclgbMatrix m, vclgbMatrix *out) {
  return convert(h, m, out, [&](Backend &be, Matrix &mm) { return convert_f32(be, mm); });
}

VCLGB_API vclgbStatus vclgbEllWrap(vclgbBackend h, vclgbPrecision prec, uint32_t rows,
                                   uint32_t cols, uint32_t width, const uint32_t *coords,
                                   const void *elems, vclgbMatrix *out) {
  if (!h || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(prec == VCLGB_FLOAT32 || prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "bad precision");
    require(!((size_t)rows * width) || (coords && elems), VCLGB_INVALID_ARGUMENT, "NULL arrays");
    auto m = std::make_unique<Matrix>();
    m->format = VCLGB_ELL;
    m->prec = prec;
    m->rows = rows;
    m->cols = cols;
    m->ell_width = width;
    m->nnz = (uint64_t)rows * width;
    m->ell_coords.borrow(coords, (size_t)rows * width * 4);
    m->ell_elems.borrow(elems, (size_t)rows * width * m->vsize());
    *out = reinterpret_cast<vclgbMatrix>(m.release());
  });
}

VCLGB_API vclgbStatus vclgbSellWrap(vclgbBackend h, vclgbPrecision prec, uint32_t rows,
                                    uint32_t cols, uint32_t C, const uint32_t *cpb,
                                    const uint32_t *colidx, const uint32_t *start,
                                    const void *elems, vclgbMatrix *out) {
  if (!h || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(prec == VCLGB_FLOAT32 || prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "bad precision");
    require(C > 0, VCLGB_INVALID_ARGUMENT, "slice height must be positive");
    auto m = std::make_unique<Matrix>();
    m->format = VCLGB_SELL;
    m->prec = prec;
    m->rows = rows;
    m->cols = cols;
    m->C = C;
    m->sigma = 1;
    if (rows) {
      require(cpb && colidx && start && elems, VCLGB_INVALID_ARGUMENT, "NULL arrays");
      uint32_t ns = (rows - 1) / C + 1;
      uint32_t last[2] = {0, 0};
      VCLGB_CUDA(cudaMemcpyAsync(&last[0], start + ns - 1, 4, cudaMemcpyDeviceToHost, be->stream));
      VCLGB_CUDA(cudaMemcpyAsync(&last[1], cpb + ns - 1, 4, cudaMemcpyDeviceToHost, be->stream));
      VCLGB_CUDA(cudaStreamSynchronize(be->stream));
      m->num_slices = ns;
      m->sell_stored = (uint64_t)last[0] + (uint64_t)last[1] * C;
      m->nnz = m->sell_stored;
      m->sell_cpb.borrow(cpb, (size_t)ns * 4);
      m->sell_start.borrow(start, (size_t)ns * 4);
      m->sell_cols.borrow(colidx, m->sell_stored * 4);
      m->sell_elems.borrow(elems, m->sell_stored * m->vsize());
      sell_wide_chunks(*be, *m);
    }
    *out = reinterpret_cast<vclgbMatrix>(m.release());
  });
}

VCLGB_API vclgbStatus vclgbHybWrap(vclgbBackend h, vclgbPrecision prec, uint32_t rows,
                                   uint32_t cols, uint32_t width, const uint32_t *ec,
                                   const void *ee, const uint32_t *trp, const uint32_t *tci,
                                   const void *tv, uint64_t tnnz, vclgbMatrix *out) {
  if (!h || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(prec == VCLGB_FLOAT32 || prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "bad precision");
    require(trp != nullptr, VCLGB_INVALID_ARGUMENT, "tail row_ptr is NULL");
    require(!tnnz || (tci && tv), VCLGB_INVALID_ARGUMENT, "NULL tail arrays");
    auto m = std::make_unique<Matrix>();
    m->format = VCLGB_HYB;
    m->prec = prec;
    m->rows = rows;
    m->cols = cols;
    m->ell_width = width;
    m->nnz = (uint64_t)rows * width + tnnz;
    m->ell_coords.borrow(ec, (size_t)rows * width * 4);
    m->ell_elems.borrow(ee, (size_t)rows * width * m->vsize());
    m->tail_nnz = tnnz;
    m->tail_rp.borrow(trp, ((size_t)rows + 1) * 4);
    m->tail_ci.borrow(tci, std::max<uint64_t>(tnnz, 1) * 4);
    m->tail_v.borrow(tv, std::max<uint64_t>(tnnz, 1) * m->vsize());
    if (tnnz) {
      m->tail_row.alloc(tnnz * 4, be->stream);
      tail_rows_from_rp(*be, rows, trp, tnnz, m->tail_row.as<uint32_t>());
      VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    }
    *out = reinterpret_cast<vclgbMatrix>(m.release());
  });
}

VCLGB_API vclgbStatus vclgbCooWrap(vclgbBackend h, vclgbPrecision prec, uint32_t rows,
                                   uint32_t cols, uint64_t nnz, const uint32_t *coords,
                                   const void *elems, vclgbMatrix *out) {
  if (!h || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(prec == VCLGB_FLOAT32 || prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "bad precision");
    require(!nnz || (coords && elems), VCLGB_INVALID_ARGUMENT, "NULL arrays");
    require(((uintptr_t)coords & 7) == 0, VCLGB_INVALID_ARGUMENT,
            "COO coordinate pairs must be 8-byte aligned");
    require(nnz <= 0xffffffffull, VCLGB_INVALID_ARGUMENT, "nnz exceeds 32-bit indices");
    auto m = std::make_unique<Matrix>();
    m->format = VCLGB_COO;
    m->prec = prec;
    m->rows = rows;
    m->cols = cols;
    m->nnz = nnz;
    m->tail_nnz = nnz;
    m->coo_stored = nnz;
    if (nnz) {
      m->coo_coords.borrow(coords, nnz * 8);
      m->coo_elems.borrow(elems, nnz * m->vsize());
      coo_validate(*be, *m);
    }
    coo_groups(*be, *m);
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbMatrix>(m.release());
  });
}

VCLGB_API vclgbStatus vclgbReadMatrixMarket(vclgbBackend h, const char *path, int64_t index_base,
                                            vclgbPrecision prec, vclgbMatrix *out,
                                            uint64_t *lines_read) {
  if (!h || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(prec == VCLGB_FLOAT32 || prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "bad precision");
    auto m = read_matrix_market(*be, path, (long)index_base, prec, lines_read);
    *out = reinterpret_cast<vclgbMatrix>(m.release());
  });
}

VCLGB_API vclgbStatus vclgbWriteMatrixMarket(vclgbBackend h, vclgbMatrix A, const char *path,
                                             int64_t index_base, int digits) {
  if (!h || !A) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { write_matrix_market(*be, *M(A), path, (long)index_base, digits); });
}

VCLGB_API vclgbStatus vclgbCuthillMcKee(vclgbBackend h, vclgbMatrix A, int advanced,
                                        double starting_node_param, uint64_t max_root_nodes,
                                        uint32_t *d_perm) {
  if (!h || !A) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    cuthill_mckee_perm(*be, *M(A), advanced != 0, starting_node_param, max_root_nodes, d_perm);
  });
}

VCLGB_API vclgbStatus vclgbCsrPermute(vclgbBackend h, vclgbMatrix A, const uint32_t *d_perm,
                                      vclgbMatrix *out) {
  if (!h || !A || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    *out = reinterpret_cast<vclgbMatrix>(csr_permute(*be, *M(A), d_perm).release());
  });
}

VCLGB_API vclgbStatus vclgbCsrBandwidth(vclgbBackend h, vclgbMatrix A, uint32_t *bandwidth) {
  if (!h || !A || !bandwidth) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { *bandwidth = csr_bandwidth(*be, *M(A)); });
}

VCLGB_API vclgbStatus vclgbMatrixDestroy(vclgbMatrix *m) {
  if (!m || !*m) return VCLGB_INVALID_ARGUMENT;
  Matrix *mm = M(*m);
  cudaDeviceSynchronize();
  FreesAfterDeviceSync legacy_frees;
  delete mm;
  *m = nullptr;
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbMatrixGetInfo(vclgbMatrix h, vclgbMatrixInfo *info) {
  if (!h || !info) return VCLGB_INVALID_ARGUMENT;
  const Matrix &m = *M(h);
  std::memset(info, 0, sizeof(*info));
  info->format = m.format;
  info->precision = m.prec;
  info->rows = m.rows;
  info->cols = m.cols;
  info->nnz = m.nnz;
  switch (m.format) {
    case VCLGB_CSR: info->stored = m.nnz; info->num_bins = m.num_bins; break;
    case VCLGB_ELL: info->stored = (uint64_t)m.rows * m.ell_width; info->ell_width = m.ell_width; break;
    case VCLGB_SELL:
      info->stored = m.sell_stored;
      info->slice_height = m.C;
      info->sigma = m.sigma;
      info->num_slices = m.num_slices;
      break;
    case VCLGB_HYB:
      info->stored = (uint64_t)m.rows * m.ell_width;
      info->ell_width = m.ell_width;
      info->tail_nnz = m.tail_nnz ? m.tail_nnz : 1;
      break;
    case VCLGB_COO: info->stored = m.coo_stored; break;
  }
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbCsrRowBlockCount(vclgbBackend h, vclgbMatrix csr, uint32_t *count) {
  if (!h || !csr || !count) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    require(M(csr)->format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "not a CSR matrix");
    csr_row_blocks(*be, *M(csr));
    *count = M(csr)->num_row_blocks;
  });
}

VCLGB_API vclgbStatus vclgbMatrixExport(vclgbBackend h, vclgbMatrix mh, int which, void *dst) {
  if (!h || !mh || !dst) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    Matrix &m = *M(mh);
    const void *src = nullptr;
    size_t bytes = 0;
    const size_t vs = m.vsize();
    switch (m.format) {
      case VCLGB_CSR:
        if (which == 0) { src = m.row_ptr; bytes = ((size_t)m.rows + 1) * 4; }
        else if (which == 1) { src = m.col_idx; bytes = m.nnz * 4; }
        else if (which == 2) { src = m.values; bytes = m.nnz * vs; }
        else if (which == 3) {
          csr_row_blocks(*be, m);
          src = m.row_blocks.ptr;
          bytes = ((size_t)m.num_row_blocks + 1) * 4;
        }
        break;
      case VCLGB_ELL:
        if (which == 0) { src = m.ell_coords.ptr; bytes = (size_t)m.rows * m.ell_width * 4; }
        else if (which == 1) { src = m.ell_elems.ptr; bytes = (size_t)m.rows * m.ell_width * vs; }
        break;
      case VCLGB_SELL:
        if (which == 0) { src = m.sell_cpb.ptr; bytes = (size_t)m.num_slices * 4; }
        else if (which == 1) { src = m.sell_cols.ptr; bytes = m.sell_stored * 4; }
        else if (which == 2) { src = m.sell_start.ptr; bytes = (size_t)m.num_slices * 4; }
        else if (which == 3) { src = m.sell_elems.ptr; bytes = m.sell_stored * vs; }
        else if (which == 4) {
          if (m.sigma > 1) { src = m.sell_perm.ptr; bytes = (size_t)m.rows * 4; }
          else {
            std::vector<uint32_t> id(m.rows);
            for (uint32_t i = 0; i < m.rows; ++i) id[i] = i;
            VCLGB_CUDA(cudaMemcpyAsync(dst, id.data(), id.size() * 4, cudaMemcpyHostToDevice, be->stream));
            VCLGB_CUDA(cudaStreamSynchronize(be->stream));
            return;
          }
        }
        break;
      case VCLGB_HYB: {
        size_t t = m.tail_nnz ? m.tail_nnz : 1;
        if (which == 0) { src = m.ell_coords.ptr; bytes = (size_t)m.rows * m.ell_width * 4; }
        else if (which == 1) { src = m.ell_elems.ptr; bytes = (size_t)m.rows * m.ell_width * vs; }
        else if (which == 2) { src = m.tail_rp.ptr; bytes = ((size_t)m.rows + 1) * 4; }
        else if (which == 3) { src = m.tail_ci.ptr; bytes = t * 4; }
        else if (which == 4) { src = m.tail_v.ptr; bytes = t * vs; }
        break;
      }
      case VCLGB_COO:
        if (which == 0) { src = m.coo_coords.ptr; bytes = m.coo_stored * 8; }
        else if (which == 1) { src = m.coo_elems.ptr; bytes = m.coo_stored * vs; }
        else if (which == 2) { src = m.coo_groups.ptr; bytes = 65 * 4; }
        break;
    }
    require(which >= 0 && (src != nullptr || bytes == 0) && which <= 4, VCLGB_INVALID_ARGUMENT,
            "no such array for this format");
    if (bytes)
      VCLGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, be->stream));
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
  });
}

VCLGB_API vclgbStatus vclgbSpmv(vclgbBackend h, vclgbMatrix A, double alpha, const void *x,
                                int64_t xs, int64_t xinc, double beta, void *y, int64_t ys,
                                int64_t yinc) {
  if (!h || !A) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    Matrix &m = *M(A);
    require(m.rows == 0 || (x && y), VCLGB_INVALID_ARGUMENT, "x or y is NULL");
    if (m.rows == 0) return;
    Reduction red{be->red_partials.ptr, be->red_counter.as<unsigned>()};
    DevBuf hyb;
    if (hyb_scratch_bytes(m)) hyb.alloc(hyb_scratch_bytes(m), be->stream);
    const bool unit = ys == 0 && yinc == 1;
    if (m.prec == VCLGB_FLOAT64) {
      with_axpby_mode(alpha, beta, [&](auto mode) {
        auto go = [&](auto e) {
          e.alpha = alpha; e.beta = beta; e.y = static_cast<double *>(y); e.ys = ys; e.yinc = yinc;
          spmv_launch<double>(*be, m, static_cast<const double *>(x), xs, xinc, e, red,
                              static_cast<double *>(y), ys, yinc, alpha, beta, nullptr, hyb.ptr);
        };
        if (unit) go(EpiAxpbyM<double, decltype(mode)::value, true>{});
        else go(EpiAxpbyM<double, decltype(mode)::value, false>{});
      });
    } else {
      const float af = (float)alpha, bf = (float)beta;
      with_axpby_mode(af, bf, [&](auto mode) {
        auto go = [&](auto e) {
          e.alpha = af; e.beta = bf; e.y = static_cast<float *>(y); e.ys = ys; e.yinc = yinc;
          spmv_launch<float>(*be, m, static_cast<const float *>(x), xs, xinc, e, red,
                             static_cast<float *>(y), ys, yinc, af, bf, nullptr, hyb.ptr);
        };
        if (unit) go(EpiAxpbyM<float, decltype(mode)::value, true>{});
        else go(EpiAxpbyM<float, decltype(mode)::value, false>{});
      });
    }
  });
}

VCLGB_API vclgbStatus vclgbDot(vclgbBackend h, vclgbPrecision prec, uint64_t n, const void *x,
                               int64_t xs, int64_t xinc, const void *y, int64_t ys, int64_t yinc,
                               void *d_result) {
  if (!h || !d_result) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { dot_launch(*be, prec, n, x, xs, xinc, y, ys, yinc, d_result, false); });
}

VCLGB_API vclgbStatus vclgbNorm2(vclgbBackend h, vclgbPrecision prec, uint64_t n, const void *x,
                                 int64_t xs, int64_t xinc, void *d_result) {
  if (!h || !d_result) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { dot_launch(*be, prec, n, x, xs, xinc, x, xs, xinc, d_result, true); });
}

// ---------------------------------------------------------------------------
VCLGB_API vclgbStatus vclgbJacobiCreate(vclgbBackend h, vclgbMatrix A, vclgbPrecond *out) {
  if (!h || !A || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    auto P = jacobi_create(*be, *M(A));
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbPrecond>(P.release());
  });
}

VCLGB_API vclgbStatus vclgbRowScalingCreate(vclgbBackend h, vclgbMatrix A, uint32_t norm,
                                            vclgbPrecond *out) {
  if (!h || !A || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    auto P = row_scaling_create(*be, *M(A), norm);
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbPrecond>(P.release());
  });
}

VCLGB_API vclgbStatus vclgbIlu0Create(vclgbBackend h, vclgbMatrix A, int lvl, vclgbPrecond *out) {
  if (!h || !A || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    auto P = ilu0_create(*be, *M(A), lvl != 0);
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbPrecond>(P.release());
  });
}

VCLGB_API vclgbStatus vclgbBlockIlu0Create(vclgbBackend h, vclgbMatrix A, uint32_t num_blocks,
                                           const uint32_t *h_bounds, vclgbPrecond *out) {
  if (!h || !A || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    auto P = block_ilu0_create(*be, *M(A), num_blocks, h_bounds);
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbPrecond>(P.release());
  });
}

static vclgbStatus chow_patel_create_api(vclgbBackend h, vclgbMatrix A, bool icc, uint32_t sweeps,
                                         uint32_t iters, vclgbPrecond *out) {
  if (!h || !A || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    auto P = chow_patel_create(*be, *M(A), icc, sweeps, iters);
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
    *out = reinterpret_cast<vclgbPrecond>(P.release());
  });
}

VCLGB_API vclgbStatus vclgbChowPatelIluCreate(vclgbBackend h, vclgbMatrix A, uint32_t sweeps,
                                              uint32_t iters, vclgbPrecond *out) {
  return chow_patel_create_api(h, A, false, sweeps, iters, out);
}

VCLGB_API vclgbStatus vclgbChowPatelIccCreate(vclgbBackend h, vclgbMatrix A, uint32_t sweeps,
                                              uint32_t iters, vclgbPrecond *out) {
  return chow_patel_create_api(h, A, true, sweeps, iters, out);
}

VCLGB_API vclgbStatus vclgbChowPatelGetInfo(vclgbPrecond p, vclgbChowPatelInfo *info) {
  if (!p || !info) return VCLGB_INVALID_ARGUMENT;
  const Precond &P = *vclgb::P(p);
  if (P.kind != 3 && P.kind != 4) return VCLGB_INVALID_ARGUMENT;
  info->kind = P.kind == 4 ? 1u : 0u;
  info->sweeps = P.sweeps;
  info->jacobi_iters = P.jacobi_iters;
  info->nnz_L = P.cp_l->nnz;
  info->nnz_U = P.cp_u->nnz;
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbChowPatelExport(vclgbBackend h, vclgbPrecond p, int which, void *dst) {
  if (!h || !p || !dst) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    const Precond &P = *vclgb::P(p);
    require(P.kind == 3 || P.kind == 4, VCLGB_INVALID_ARGUMENT, "not a Chow-Patel preconditioner");
    require(which >= 0 && which <= 7, VCLGB_INVALID_ARGUMENT, "no such Chow-Patel array");
    const Matrix &m = which < 4 ? *P.cp_l : *P.cp_u;
    const size_t vs = P.prec == VCLGB_FLOAT64 ? 8 : 4;
    const void *src = nullptr;
    size_t bytes = 0;
    switch (which & 3) {
      case 0: src = m.row_ptr; bytes = ((size_t)P.rows + 1) * 4; break;
      case 1: src = m.col_idx; bytes = m.nnz * 4; break;
      case 2: src = m.values; bytes = m.nnz * vs; break;
      default: src = which < 4 ? P.diag.ptr : P.diag_u.ptr; bytes = (size_t)P.rows * vs; break;
    }
    if (bytes) VCLGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, be->stream));
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
  });
}

VCLGB_API vclgbStatus vclgbPrecondApply(vclgbBackend h, vclgbPrecond P, void *vec) {
  if (!h || !P || !vec) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { precond_apply(*be, *vclgb::P(P), vec, nullptr); });
}

VCLGB_API vclgbStatus vclgbMatrixAutotune(vclgbBackend h, vclgbMatrix A, vclgbTuneInfo *info) {
  if (!h || !A || !info) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { matrix_autotune(*be, *M(A), info); });
}

VCLGB_API vclgbStatus vclgbMatrixAutotuneClear(vclgbMatrix A) {
  if (!A) return VCLGB_INVALID_ARGUMENT;
  return guarded(nullptr, [&]() {
    cudaDeviceSynchronize();  // no product may still read the tuned form
    M(A)->tuned.reset();
  });
}

VCLGB_API vclgbStatus vclgbCsrInplaceSolve(vclgbBackend h, vclgbMatrix A, int tag, int transposed,
                                           void *vec) {
  if (!h || !A || !vec) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { csr_inplace_solve(*be, *M(A), tag, transposed != 0, vec); });
}

VCLGB_API vclgbStatus vclgbPrecondDestroy(vclgbPrecond *p) {
  if (!p || !*p) return VCLGB_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  FreesAfterDeviceSync legacy_frees;
  delete vclgb::P(*p);
  *p = nullptr;
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbIlu0GetInfo(vclgbPrecond p, vclgbIlu0Info *info) {
  if (!p || !info || vclgb::P(p)->kind != 2) return VCLGB_INVALID_ARGUMENT;
  const Precond &P = *vclgb::P(p);
  info->num_levels_L = P.L.levels;
  info->num_levels_U = P.U.levels;
  info->rows_L = P.L.rows;
  info->rows_U = P.U.rows;
  info->nnz_L = P.L.nnz;
  info->nnz_U = P.U.nnz;
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbIlu0Export(vclgbBackend h, vclgbPrecond p, int which, void *dst) {
  if (!h || !p || !dst) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    const Precond &P = *vclgb::P(p);
    require(P.kind == 2, VCLGB_INVALID_ARGUMENT, "not an ILU0 preconditioner");
    size_t vs = P.prec == VCLGB_FLOAT64 ? 8 : 4;
    const void *src = nullptr;
    size_t bytes = 0;
    const Precond::Tri &t = which >= 7 ? P.U : P.L;
    int w = which >= 7 ? which - 5 : which;
    switch (w) {
      case 0: src = P.lu.ptr; bytes = P.nnz * vs; break;
      case 1: src = P.diag.ptr; bytes = (size_t)P.rows * vs; break;
      case 2: src = t.level_ptr.ptr; bytes = ((size_t)t.levels + 1) * 4; break;
      case 3: src = t.row_index.ptr; bytes = t.rows * 4; break;
      case 4: src = t.row_ptr.ptr; bytes = (t.rows + 1) * 4; break;
      case 5: src = t.cols.ptr; bytes = t.nnz * 4; break;
      case 6: src = t.vals.ptr; bytes = t.nnz * vs; break;
      default: throw Error(VCLGB_INVALID_ARGUMENT, "no such ILU0 array");
    }
    if (bytes) VCLGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, be->stream));
    VCLGB_CUDA(cudaStreamSynchronize(be->stream));
  });
}

// ---------------------------------------------------------------------------
static bool bad_vec(const void *p, int64_t start, int64_t stride, uint64_t n) {
  return n && (!p || start < 0 || stride == 0);
}

VCLGB_API vclgbStatus vclgbAvbv(vclgbBackend h, vclgbPrecision prec, uint64_t n, void *y,
                                int64_t ys, int64_t yinc, const void *x, int64_t xs, int64_t xinc,
                                vclgbScalarArg alpha, const void *z, int64_t zs, int64_t zinc,
                                vclgbScalarArg beta, int accumulate) {
  if (!h || bad_vec(y, ys, yinc, n) || bad_vec(x, xs, xinc, n) || (z && bad_vec(z, zs, zinc, n)))
    return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    const VecArg vy{y, ys, yinc}, vx{x, xs, xinc}, vz{z, zs, zinc};
    avbv(*be, prec, n, vy, vx, alpha, z ? &vz : nullptr, z ? &beta : nullptr, accumulate != 0);
  });
}

VCLGB_API vclgbStatus vclgbElementBinary(vclgbBackend h, vclgbPrecision prec, uint64_t n, void *y,
                                         int64_t ys, int64_t yinc, const void *x, int64_t xs,
                                         int64_t xinc, vclgbScalarArg xsc, const void *z,
                                         int64_t zs, int64_t zinc, vclgbScalarArg zsc, int op) {
  if (!h || bad_vec(y, ys, yinc, n) || (x && bad_vec(x, xs, xinc, n)) ||
      (z && bad_vec(z, zs, zinc, n)))
    return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    const VecArg vy{y, ys, yinc}, vx{x, xs, xinc}, vz{z, zs, zinc};
    element_binary(*be, prec, n, vy, x ? &vx : nullptr, xsc, z ? &vz : nullptr, zsc, op);
  });
}

VCLGB_API vclgbStatus vclgbElementUnary(vclgbBackend h, vclgbPrecision prec, uint64_t n, void *y,
                                        int64_t ys, int64_t yinc, const void *x, int64_t xs,
                                        int64_t xinc, int op) {
  if (!h || bad_vec(y, ys, yinc, n) || bad_vec(x, xs, xinc, n)) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { element_unary(*be, prec, n, {y, ys, yinc}, {x, xs, xinc}, op); });
}

VCLGB_API vclgbStatus vclgbVectorAssign(vclgbBackend h, vclgbPrecision prec, uint64_t n, void *y,
                                        int64_t ys, int64_t yinc, double alpha) {
  if (!h || bad_vec(y, ys, yinc, n)) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { vector_assign(*be, prec, n, {y, ys, yinc}, alpha); });
}

VCLGB_API vclgbStatus vclgbVectorSwap(vclgbBackend h, vclgbPrecision prec, uint64_t n, void *x,
                                      int64_t xs, int64_t xinc, void *y, int64_t ys, int64_t yinc) {
  if (!h || bad_vec(x, xs, xinc, n) || bad_vec(y, ys, yinc, n)) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { vector_swap(*be, prec, n, {x, xs, xinc}, {y, ys, yinc}); });
}

// ---------------------------------------------------------------------------
VCLGB_API void vclgbSolverTagInit(vclgbSolverTag *t, int kind) {
  if (!t) return;
  std::memset(t, 0, sizeof(*t));
  if (kind == 1) { t->tol = 1e-8; t->max_iters = 400; t->max_iters_before_restart = 200; }
  else if (kind == 2) { t->tol = 1e-10; t->max_iters = 300; t->krylov_dim = 20; }
  else { t->tol = 1e-8; t->max_iters = 300; }
}

VCLGB_API vclgbStatus vclgbSolveCG(vclgbBackend h, vclgbMatrix A, const void *b, void *x,
                                   vclgbSolverTag *tag, vclgbPrecond P) {
  return solve_entry(h, A, b, x, tag, [&](Backend &be, Matrix &m) {
    if (m.prec == VCLGB_FLOAT64)
      cg_solve<double>(be, m, static_cast<const double *>(b), static_cast<double *>(x), tag,
                       P ? vclgb::P(P) : nullptr);
    else
      cg_solve<float>(be, m, static_cast<const float *>(b), static_cast<float *>(x), tag,
                      P ? vclgb::P(P) : nullptr);
  });
}

VCLGB_API vclgbStatus vclgbSolveBiCGStab(vclgbBackend h, vclgbMatrix A, const void *b, void *x,
                                         vclgbSolverTag *tag, vclgbPrecond P) {
  return solve_entry(h, A, b, x, tag, [&](Backend &be, Matrix &m) {
    if (m.prec == VCLGB_FLOAT64)
      bicgstab_solve<double>(be, m, static_cast<const double *>(b), static_cast<double *>(x), tag,
                             P ? vclgb::P(P) : nullptr);
    else
      bicgstab_solve<float>(be, m, static_cast<const float *>(b), static_cast<float *>(x), tag,
                            P ? vclgb::P(P) : nullptr);
  });
}

VCLGB_API vclgbStatus vclgbSolveGMRES(vclgbBackend h, vclgbMatrix A, const void *b, void *x,
                                      vclgbSolverTag *tag, vclgbPrecond P) {
  return solve_entry(h, A, b, x, tag, [&](Backend &be, Matrix &m) {
    if (m.prec == VCLGB_FLOAT64)
      gmres_solve<double>(be, m, static_cast<const double *>(b), static_cast<double *>(x), tag,
                          P ? vclgb::P(P) : nullptr);
    else
      gmres_solve<float>(be, m, static_cast<const float *>(b), static_cast<float *>(x), tag,
                         P ? vclgb::P(P) : nullptr);
  });
}

VCLGB_API vclgbStatus vclgbSolveMixedCG(vclgbBackend h, vclgbMatrix A, const void *b, void *x,
                                        vclgbSolverTag *tag, float inner_tol) {
  return solve_entry(h, A, b, x, tag, [&](Backend &be, Matrix &m) {
    require(m.prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "mixed CG takes an FP64 matrix");
    mixed_cg_solve(be, m, static_cast<const double *>(b), static_cast<double *>(x), tag, inner_tol);
  });
}

VCLGB_API vclgbStatus vclgbSolveRefinedCG(vclgbBackend h, vclgbMatrix A, const void *b, void *x,
                                          vclgbSolverTag *tag, double inner_tol,
                                          uint32_t max_outer, uint32_t *outer_iters) {
  return solve_entry(h, A, b, x, tag, [&](Backend &be, Matrix &m) {
    require(m.prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT, "refined CG takes an FP64 matrix");
    refined_cg_solve(be, m, static_cast<const double *>(b), static_cast<double *>(x), tag,
                     inner_tol, max_outer, outer_iters);
  });
}

// ---------------------------------------------------------------------------
VCLGB_API vclgbStatus vclgbBatchCreate(vclgbBackend h, vclgbMatrix A, uint32_t nsys,
                                       const uint32_t *h_sys_ptr, const int32_t *h_methods,
                                       vclgbBatch *out) {
  if (!h || !A || !out) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    Batch *bt = batch_create(*be, *M(A), nsys, h_sys_ptr, h_methods);
    *out = reinterpret_cast<vclgbBatch>(bt);
  });
}

VCLGB_API vclgbStatus vclgbBatchTune(vclgbBackend h, vclgbBatch bt, const void *b, int32_t *block,
                                     int32_t *lanes) {
  if (!h || !bt || !b) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() {
    Batch &batch = *reinterpret_cast<Batch *>(bt);
    batch_tune(*be, batch, static_cast<const double *>(b));
    int bb = 0, ll = 0;
    batch_config(batch, &bb, &ll);
    if (block) *block = bb;
    if (lanes) *lanes = ll;
  });
}

VCLGB_API vclgbStatus vclgbBatchSolve(vclgbBackend h, vclgbBatch bt, const void *b, void *x,
                                      double tol, uint32_t max_iters, uint32_t *h_iters,
                                      int32_t *h_status, double *h_error) {
  if (!h || !bt || !b || !x) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  Batch &batch = *reinterpret_cast<Batch *>(bt);
  bool all = false;
  vclgbStatus s = guarded(be, [&]() {
    all = batch_solve(*be, batch, static_cast<const double *>(b), static_cast<double *>(x), tol,
                      max_iters, h_iters, h_status, h_error);
  });
  if (s != VCLGB_SUCCESS) return s;
  return all ? VCLGB_SUCCESS : VCLGB_NOT_CONVERGED;
}

VCLGB_API vclgbStatus vclgbBatchDestroy(vclgbBatch *bt) {
  if (!bt || !*bt) return VCLGB_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  FreesAfterDeviceSync legacy_frees;
  batch_destroy(reinterpret_cast<Batch *>(*bt));
  *bt = nullptr;
  return VCLGB_SUCCESS;
}

VCLGB_API vclgbStatus vclgbSolveAdjoint(vclgbBackend h, vclgbMatrix A, int solver, vclgbPrecond P,
                                        const void *x, const void *dLdx, void *dLdb, void *dLdA,
                                        vclgbSolverTag *tag, int symmetric) {
  if (!h || !A || !x || !dLdx || !dLdb || !tag) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  vclgbStatus s = guarded(be, [&]() {
    Matrix &m = *M(A);
    const Precond *pc = P ? vclgb::P(P) : nullptr;
    if (m.prec == VCLGB_FLOAT64)
      adjoint_solve<double>(*be, m, solver, pc, static_cast<const double *>(x),
                            static_cast<const double *>(dLdx), static_cast<double *>(dLdb),
                            static_cast<double *>(dLdA), tag, symmetric != 0);
    else
      adjoint_solve<float>(*be, m, solver, pc, static_cast<const float *>(x),
                           static_cast<const float *>(dLdx), static_cast<float *>(dLdb),
                           static_cast<float *>(dLdA), tag, symmetric != 0);
  });
  if (s != VCLGB_SUCCESS) {
    tag->status = s;
    return s;
  }
  return (vclgbStatus)tag->status;
}

VCLGB_API vclgbStatus vclgbTransposeExport(vclgbBackend h, vclgbMatrix A, int which, void *dst) {
  if (!h || !A || !dst) return VCLGB_INVALID_ARGUMENT;
  Backend *be = B(h);
  return guarded(be, [&]() { transpose_export(*be, *M(A), which, dst); });
}

}  // extern "C"
