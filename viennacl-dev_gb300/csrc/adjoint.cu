// adjoint.cu -- backward pass of a linear solve (no reference counterpart).
//
// For x = A^-1 b and a loss L(x):  A^T lambda = dL/dx,  dL/db = lambda,
// dL/dA_ij = -lambda_i x_j on the sparsity pattern of A.  A^T is built once on
// the device together with a map from each transposed entry to its position
// in A (so new values on the same pattern only need a gather), then cached on
// A.  The adjoint solve reuses the Krylov solvers; the gradient on the
// pattern is one fused kernel.  Only x from the forward solve is stored.
#include <algorithm>

#include "formats.hpp"
#include "vecpass.cuh"

namespace vclgb {

template <typename T>
void cg_solve(Backend &, Matrix &, const T *, T *, vclgbSolverTag *, const Precond *);
template <typename T>
void bicgstab_solve(Backend &, Matrix &, const T *, T *, vclgbSolverTag *, const Precond *);
template <typename T>
void gmres_solve(Backend &, Matrix &, const T *, T *, vclgbSolverTag *, const Precond *);

__global__ void col_count_kernel(uint64_t nnz, const uint32_t *__restrict__ ci, uint32_t *cnt) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (size_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[ci[k]], 1u);
}

__global__ void t_scatter_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                 const uint32_t *__restrict__ ci, uint32_t *cursor, uint32_t *tci,
                                 uint32_t *map) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x)
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k) {
      uint32_t pos = atomicAdd(&cursor[ci[k]], 1u);
      tci[pos] = (uint32_t)r;
      map[pos] = k;
    }
}

// rows inside each transposed row in ascending order (deterministic layout);
// (row, map) pairs move together; an entry's map is unique, so ties cannot occur
__global__ void t_sort_kernel(uint32_t cols, const uint32_t *__restrict__ trp, uint32_t *tci,
                              uint32_t *map) {
  for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < cols;
       c += (size_t)gridDim.x * blockDim.x) {
    uint32_t s = trp[c], e = trp[c + 1];
    for (uint32_t i = s + 1; i < e; ++i) {
      uint32_t kr = tci[i], km = map[i];
      uint32_t j = i;
      while (j > s && (tci[j - 1] > kr || (tci[j - 1] == kr && map[j - 1] > km))) {
        tci[j] = tci[j - 1];
        map[j] = map[j - 1];
        --j;
      }
      tci[j] = kr;
      map[j] = km;
    }
  }
}

template <typename W>
__global__ void t_gather_kernel(uint64_t nnz, const uint32_t *__restrict__ map,
                                const W *__restrict__ v, W *tv) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (size_t)gridDim.x * blockDim.x)
    tv[k] = v[map[k]];
}

struct Transposed {
  std::unique_ptr<Matrix> T;
  DevBuf map;
};

void csr_transpose_pattern(Backend &be, uint32_t rows, uint32_t cols, uint64_t nnz,
                           const uint32_t *rp, const uint32_t *ci, DevBuf &trp, DevBuf &tci,
                           DevBuf &map) {
  trp.alloc(((size_t)cols + 1) * 4, be.stream);
  tci.alloc(std::max<uint64_t>(nnz, 1) * 4, be.stream);
  map.alloc(std::max<uint64_t>(nnz, 1) * 4, be.stream);
  DevBuf cnt(std::max<size_t>(cols, 1) * 4, be.stream);
  VCLGB_CUDA(cudaMemsetAsync(cnt.ptr, 0, cnt.bytes, be.stream));
  int g = waves_grid(be, 256, 8, std::max<uint64_t>(nnz, 1));
  col_count_kernel<<<g, 256, 0, be.stream>>>(nnz, ci, cnt.as<uint32_t>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  extern_scan_u32(be, cnt.as<uint32_t>(), cols, trp.as<uint32_t>());
  DevBuf cursor(std::max<size_t>(cols, 1) * 4, be.stream);
  VCLGB_CUDA(cudaMemcpyAsync(cursor.ptr, trp.ptr, (size_t)cols * 4, cudaMemcpyDeviceToDevice,
                             be.stream));
  int gr = waves_grid(be, 256, 8, rows);
  t_scatter_kernel<<<gr, 256, 0, be.stream>>>(rows, rp, ci, cursor.as<uint32_t>(),
                                              tci.as<uint32_t>(), map.as<uint32_t>());
  int gc = waves_grid(be, 256, 8, cols);
  t_sort_kernel<<<gc, 256, 0, be.stream>>>(cols, trp.as<uint32_t>(), tci.as<uint32_t>(),
                                           map.as<uint32_t>());
  be.launches += 2;
  VCLGB_CHECK_LAUNCH();
}

static Transposed &transpose_of(Backend &be, Matrix &A) {
  static_assert(sizeof(Transposed) > 0, "");
  if (A.transposed) return *A.transposed;
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "the adjoint needs a CSR matrix");
  auto tr = std::make_unique<Transposed>();
  auto m = std::make_unique<Matrix>();
  m->format = VCLGB_CSR;
  m->prec = A.prec;
  m->rows = A.cols;
  m->cols = A.rows;
  m->nnz = A.nnz;
  csr_transpose_pattern(be, A.rows, A.cols, A.nnz, A.row_ptr, A.col_idx, m->own_row_ptr,
                        m->own_col_idx, tr->map);
  m->own_values.alloc(std::max<uint64_t>(A.nnz, 1) * A.vsize(), be.stream);
  int g = waves_grid(be, 256, 8, std::max<uint64_t>(A.nnz, 1));
  if (A.vsize() == 8)
    t_gather_kernel<uint64_t><<<g, 256, 0, be.stream>>>(
        A.nnz, tr->map.as<uint32_t>(), static_cast<const uint64_t *>(A.values),
        m->own_values.as<uint64_t>());
  else
    t_gather_kernel<uint32_t><<<g, 256, 0, be.stream>>>(
        A.nnz, tr->map.as<uint32_t>(), static_cast<const uint32_t *>(A.values),
        m->own_values.as<uint32_t>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  m->row_ptr = m->own_row_ptr.as<uint32_t>();
  m->col_idx = m->own_col_idx.as<uint32_t>();
  m->values = m->own_values.ptr;
  csr_analyse(be, *m);
  tr->T = std::move(m);
  A.transposed.reset(tr.release());
  return *A.transposed;
}

void transpose_export(Backend &be, Matrix &A, int which, void *dst) {
  Transposed &t = transpose_of(be, A);
  const Matrix &T = *t.T;
  const void *src = nullptr;
  size_t bytes = 0;
  if (which == 0) { src = T.row_ptr; bytes = ((size_t)T.rows + 1) * 4; }
  else if (which == 1) { src = T.col_idx; bytes = T.nnz * 4; }
  else if (which == 2) { src = T.values; bytes = T.nnz * T.vsize(); }
  else if (which == 3) { src = t.map.ptr; bytes = T.nnz * 4; }
  else throw Error(VCLGB_INVALID_ARGUMENT, "no such transpose array");
  if (bytes) VCLGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
}

// dL/dA_ij = -lambda_i x_j on A's pattern (thread per row)
template <typename T>
__global__ void pattern_grad_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                    const uint32_t *__restrict__ ci, const T *__restrict__ lam,
                                    const T *__restrict__ x, T *g) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    T l = -lam[r];
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k) g[k] = l * x[ci[k]];
  }
}

template <typename T>
void adjoint_solve(Backend &be, Matrix &A, int solver, const Precond *P, const T *x,
                   const T *dLdx, T *dLdb, T *dLdA, vclgbSolverTag *tag, bool symmetric) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "the adjoint needs a CSR matrix");
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "the adjoint needs a square matrix");
  Matrix &At = symmetric ? A : *transpose_of(be, A).T;
  // diag(A^T) = diag(A): the Jacobi preconditioner of A serves A^T unchanged
  require(!P || P->kind == 1, VCLGB_UNSUPPORTED, "the adjoint takes Jacobi or no preconditioner");
  switch (solver) {
    case 0: cg_solve<T>(be, At, dLdx, dLdb, tag, P); break;
    case 1: bicgstab_solve<T>(be, At, dLdx, dLdb, tag, P); break;
    case 2: gmres_solve<T>(be, At, dLdx, dLdb, tag, P); break;
    default: throw Error(VCLGB_INVALID_ARGUMENT, "solver must be 0 (CG), 1 (BiCGStab), 2 (GMRES)");
  }
  if (dLdA) {
    int g = waves_grid(be, 256, 8, A.rows);
    pattern_grad_kernel<T><<<g, 256, 0, be.stream>>>(A.rows, A.row_ptr, A.col_idx, dLdb, x, dLdA);
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  }
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
}

template void adjoint_solve<double>(Backend &, Matrix &, int, const Precond *, const double *,
                                    const double *, double *, double *, vclgbSolverTag *, bool);
template void adjoint_solve<float>(Backend &, Matrix &, int, const Precond *, const float *,
                                   const float *, float *, float *, vclgbSolverTag *, bool);

void transposed_destroy(Transposed *t) { delete t; }

}  // namespace vclgb
