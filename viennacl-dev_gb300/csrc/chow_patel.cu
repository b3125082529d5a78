// chow_patel.cu -- Chow-Patel fine-grained parallel ILU0 / ICC0 preconditioners
// (linalg/detail/ilu/chow_patel_ilu.hpp; the kernels of
// linalg/cuda/ilu_operations.hpp and linalg/host_based/ilu_operations.hpp).
//
// Setup, all on the device: split A into L (col <= row) and U (col >= row),
// scale both by D = |diag(A)|^-1/2 on each side, run `sweeps` nonlinear
// Jacobi sweeps -- every entry is recomputed from the previous sweep's values,
// as the reference's backup copies make it, so no result depends on thread
// scheduling -- and form the Neumann matrices I - D_L^-1 L and I - D_U^-1 U.
// Every multiply, add, divide and square root is a separately rounded IEEE
// operation in the reference's order (no fused multiply-add), so the factors
// equal the reference host backend's bit for bit.
//
// A sweep is one launch with one thread per entry of L and of U^T: an entry
// merges two short sorted rows, so the work is balanced by entries, not rows.
//
// Apply: x = D^-1 v, then jacobi_iters steps x <- N x + D^-1 v per triangle.
// A step is one SpMV over the strictly triangular Neumann matrix (the zero
// diagonal the reference stores is left out) with "+ D^-1 v" -- and, closing
// the L phase, the scaling by D_U^-1 that starts the U phase -- in its
// epilogue.  The apply multiplies by reciprocals of D formed once at setup (an
// FP64 division is a long software sequence on GB300), so it agrees with the
// reference's divisions to rounding, like its fused multiply-add SpMV.
#include <algorithm>

#include "formats.hpp"
#include "vecpass.cuh"

namespace vclgb {
namespace {

template <typename T>
struct Rn;
template <>
struct Rn<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ double root(double a) { return __dsqrt_rn(a); }
};
template <>
struct Rn<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ float root(float a) { return __fsqrt_rn(a); }
};

constexpr unsigned kUnsorted = 1, kNoDiagonal = 2, kZeroDiagonal = 4;

// per row: the checks the sweeps rely on (ascending, duplicate-free columns and
// a diagonal entry), D_r = 1 / sqrt(|a_rr|) (ilu_scale, ilu_operations.hpp:348-428)
// and the lengths of the row's L and U parts (extract_LU, :257-345)
template <typename T>
__global__ void cp_rows_kernel(uint32_t n, const uint32_t *__restrict__ rp,
                               const uint32_t *__restrict__ ci, const T *__restrict__ v, T *D,
                               uint32_t *lcnt, uint32_t *ucnt, unsigned *flags) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x) {
    const uint32_t s = rp[r], e = rp[r + 1];
    uint32_t nl = 0, prev = 0;
    bool diag = false;
    T dv = T(0);
    for (uint32_t j = s; j < e; ++j) {
      const uint32_t c = ci[j];
      if (j > s && c <= prev) atomicOr(flags, kUnsorted);
      prev = c;
      if (c <= r) ++nl;
      if (c == r && !diag) {
        diag = true;
        dv = v[j];
      }
    }
    if (!diag) atomicOr(flags, kNoDiagonal);
    else if (dv == T(0)) atomicOr(flags, kZeroDiagonal);
    D[r] = diag ? Rn<T>::div(T(1), Rn<T>::root(fabs(dv))) : T(0);
    lcnt[r] = nl;
    if (ucnt) ucnt[r] = (e - s) - nl + (diag ? 1u : 0u);
  }
}

// L and U entries in storage order, scaled: m_ij * (D_i * D_j); row of each L entry
template <typename T>
__global__ void cp_split_kernel(uint32_t n, const uint32_t *__restrict__ rp,
                                const uint32_t *__restrict__ ci, const T *__restrict__ v,
                                const T *__restrict__ D, const uint32_t *__restrict__ lrp,
                                uint32_t *lci, T *lv, uint32_t *lrow,
                                const uint32_t *__restrict__ urp, uint32_t *uci, T *uv) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x) {
    const T dr = D[r];
    uint32_t kl = lrp[r], ku = urp ? urp[r] : 0u;
    for (uint32_t j = rp[r]; j < rp[r + 1]; ++j) {
      const uint32_t c = ci[j];
      const T sc = Rn<T>::mul(v[j], Rn<T>::mul(dr, D[c]));
      if (c <= r) {
        lci[kl] = c;
        lv[kl] = sc;
        lrow[kl] = (uint32_t)r;
        ++kl;
      }
      if (urp && c >= r) {
        uci[ku] = c;
        uv[ku] = sc;
        ++ku;
      }
    }
  }
}

__global__ void cp_row_of_kernel(uint32_t n, const uint32_t *__restrict__ rp, uint32_t *row_of) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x)
    for (uint32_t j = rp[r]; j < rp[r + 1]; ++j) row_of[j] = (uint32_t)r;
}

template <typename T>
__global__ void cp_gather_kernel(uint64_t nnz, const uint32_t *__restrict__ map,
                                 const T *__restrict__ src, T *dst) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (size_t)gridDim.x * blockDim.x)
    dst[k] = src[map[k]];
}

template <typename T>
__global__ void cp_scatter_kernel(uint64_t nnz, const uint32_t *__restrict__ map,
                                  const T *__restrict__ src, T *dst) {
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < nnz;
       k += (size_t)gridDim.x * blockDim.x)
    dst[map[k]] = src[k];
}

// one sweep of ilu_chow_patel_sweep (ilu_operations.hpp:502-623): entries
// [0, nl) are L's, [nl, nl + nu) U^T's; old values in Lo/Uo, new in Ln/Un.
//   l_ij = (a_ij - sum_{k<j} l_ik u_kj) / u_jj      (L's diagonal is kept)
//   u_ij =  a_ij - sum_{k<i} l_ik u_kj
// The merges walk both sorted rows exactly as the reference does; past the end
// of a row the column reads as n, which stops the walk inside the row.
template <typename T>
__global__ void cp_ilu_sweep_kernel(uint32_t n, uint64_t nl, uint64_t nu,
                                    const uint32_t *__restrict__ lrp,
                                    const uint32_t *__restrict__ lci,
                                    const uint32_t *__restrict__ lrow, const T *__restrict__ aL,
                                    const T *__restrict__ Lo, T *Ln,
                                    const uint32_t *__restrict__ utrp,
                                    const uint32_t *__restrict__ utci,
                                    const uint32_t *__restrict__ utrow, const T *__restrict__ aU,
                                    const T *__restrict__ Uo, T *Un) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nl + nu;
       t += (size_t)gridDim.x * blockDim.x) {
    if (t < nl) {
      const uint32_t j = (uint32_t)t, row = lrow[j], col = lci[j];
      if (col == row) {
        Ln[j] = Lo[j];
        continue;
      }
      uint32_t iu = utrp[col];
      const uint32_t ue = utrp[col + 1];
      uint32_t cu = iu < ue ? utci[iu] : n;
      T sum = T(0);
      for (uint32_t k = lrp[row]; k < j; ++k) {
        const uint32_t cl = lci[k];
        while (cu < cl) {
          ++iu;
          cu = iu < ue ? utci[iu] : n;
        }
        if (cu == cl) sum = Rn<T>::add(sum, Rn<T>::mul(Lo[k], Uo[iu]));
      }
      Ln[j] = Rn<T>::div(Rn<T>::sub(aL[j], sum), Uo[ue - 1]);
    } else {
      const uint32_t j = (uint32_t)(t - nl), row = utrow[j], col = utci[j];
      uint32_t il = lrp[col];
      const uint32_t le = lrp[col + 1];
      uint32_t cl = il < le ? lci[il] : n;
      T sum = T(0);
      for (uint32_t k = utrp[row]; k < j; ++k) {
        const uint32_t cu = utci[k];
        while (cl < cu) {
          ++il;
          cl = il < le ? lci[il] : n;
        }
        if (cu == cl) sum = Rn<T>::add(sum, Rn<T>::mul(Lo[il], Uo[k]));
      }
      Un[j] = Rn<T>::sub(aU[j], sum);
    }
  }
}

// one sweep of icc_chow_patel_sweep (ilu_operations.hpp:184-255):
//   l_ij = (a_ij - sum_{k<j} l_ik l_jk) / l_jj,   l_ii = sqrt(a_ii - sum_k l_ik^2)
template <typename T>
__global__ void cp_icc_sweep_kernel(uint32_t n, uint64_t nl, const uint32_t *__restrict__ lrp,
                                    const uint32_t *__restrict__ lci,
                                    const uint32_t *__restrict__ lrow, const T *__restrict__ aL,
                                    const T *__restrict__ Lo, T *Ln) {
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nl;
       t += (size_t)gridDim.x * blockDim.x) {
    const uint32_t i = (uint32_t)t, row = lrow[i], col = lci[i];
    uint32_t ij = lrp[col];
    const uint32_t je = lrp[col + 1];
    uint32_t cj = ij < je ? lci[ij] : n;
    T s = aL[i];
    for (uint32_t ii = lrp[row]; ii < i; ++ii) {
      const uint32_t c = lci[ii];
      while (cj < c) {
        ++ij;
        cj = ij < je ? lci[ij] : n;
      }
      if (cj == c) s = Rn<T>::sub(s, Rn<T>::mul(Lo[ii], Lo[ij]));
    }
    Ln[i] = col != row ? Rn<T>::div(s, Lo[je - 1]) : Rn<T>::root(s);
  }
}

// ilu_form_neumann_matrix (ilu_operations.hpp:625-667) on a triangle whose
// rows hold exactly one diagonal entry, last (lower) or first (upper): d is
// that entry, the other entries become m_ij / -d and are written without the
// diagonal -- row r of the output starts at rp[r] - r.
template <typename T>
__global__ void cp_neumann_kernel(uint32_t n, const uint32_t *__restrict__ rp,
                                  const uint32_t *__restrict__ ci, const T *__restrict__ v,
                                  bool diag_last, T *diag, uint32_t *orp, uint32_t *oci, T *ov) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (size_t)gridDim.x * blockDim.x) {
    const uint32_t s = rp[r], e = rp[r + 1];
    const T d = v[diag_last ? e - 1 : s];
    diag[r] = d;
    const T nd = -d;
    const uint32_t j0 = diag_last ? s : s + 1, j1 = diag_last ? e - 1 : e;
    uint32_t o = s - (uint32_t)r;
    orp[r] = o;
    for (uint32_t j = j0; j < j1; ++j, ++o) {
      oci[o] = ci[j];
      ov[o] = Rn<T>::div(v[j], nd);
    }
    if (r + 1 == n) orp[n] = e - n;
  }
}

// the reciprocals of D_L and D_U, formed once so that the apply multiplies
template <typename T>
__global__ void cp_recip_kernel(uint32_t n, const T *__restrict__ dl, const T *__restrict__ du,
                                T *rl, T *ru) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    rl[i] = T(1) / dl[i];
    ru[i] = T(1) / du[i];
  }
}

// b = v D_L^-1 (element_div), or (v D_L^-1) D_U^-1 when a triangle takes no
// Jacobi step; TWO is a template argument so that no path carries the other
template <typename T, bool TWO>
__global__ void cp_scale_kernel(size_t n, const T *src, const T *__restrict__ r1,
                                const T *__restrict__ r2, T *dst, const int *skip) {
  if (skip && *skip) return;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    T b = src[i] * r1[i];
    if (TWO) b = b * r2[i];
    dst[i] = b;
  }
}

}  // namespace

// x_{k+1} = N x_k + D^-1 rhs (chow_patel_ilu.hpp:281-285): out = acc + rhs,
// times D_U^-1 when the step closes the L phase (b_U = x_L / D_U).  SCALE is a
// template argument: as a runtime flag the compiler kept the scaling work in
// every step.
template <typename T, bool SCALE>
struct EpiCpStep {
  static constexpr int NDOT = 0;
  T *out; const T *rhs; const T *r; const int *flag;
  struct Pre { T rhs, r; };
  __device__ bool skip() const { return flag && *flag; }
  __device__ Pre pre(uint32_t i) const { return {rhs[i], SCALE ? r[i] : T(1)}; }
  __device__ void row(uint32_t i, T acc, const Pre &p, T (&)[1]) const {
    const T v = acc + p.rhs;
    out[i] = SCALE ? v * p.r : v;
  }
  __device__ void finalize(const T (&)[1]) const {}
};

static std::unique_ptr<Matrix> neumann_matrix(Backend &be, vclgbPrecision prec, uint32_t n,
                                              uint64_t nnz_with_diag) {
  auto m = std::make_unique<Matrix>();
  m->format = VCLGB_CSR;
  m->prec = prec;
  m->rows = m->cols = n;
  m->nnz = nnz_with_diag - n;
  m->own_row_ptr.alloc(((size_t)n + 1) * 4, be.stream);
  m->own_col_idx.alloc(std::max<uint64_t>(m->nnz, 1) * 4, be.stream);
  m->own_values.alloc(std::max<uint64_t>(m->nnz, 1) * m->vsize(), be.stream);
  m->row_ptr = m->own_row_ptr.as<uint32_t>();
  m->col_idx = m->own_col_idx.as<uint32_t>();
  m->values = m->own_values.ptr;
  if (n == 0) VCLGB_CUDA(cudaMemsetAsync(m->own_row_ptr.ptr, 0, 4, be.stream));
  return m;
}

template <typename T>
static void cp_build(Backend &be, const Matrix &A, bool icc, Precond &P) {
  const uint32_t n = A.rows;
  const size_t vs = sizeof(T);
  if (n == 0) {
    P.cp_l = neumann_matrix(be, A.prec, 0, 0);
    P.cp_u = neumann_matrix(be, A.prec, 0, 0);
    P.diag.alloc(vs, be.stream);
    P.diag_u.alloc(vs, be.stream);
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    return;
  }
  const T *av = static_cast<const T *>(A.values);
  const int g = waves_grid(be, 256, 8, n);
  // checks, D, L / U lengths
  DevBuf D(std::max<size_t>(n, 1) * sizeof(T), be.stream);
  DevBuf lcnt(std::max<size_t>(n, 1) * 4, be.stream), ucnt(std::max<size_t>(n, 1) * 4, be.stream);
  DevBuf flags(sizeof(unsigned), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(flags.ptr, 0, sizeof(unsigned), be.stream));
  cp_rows_kernel<T><<<g, 256, 0, be.stream>>>(n, A.row_ptr, A.col_idx, av, D.as<T>(),
                                              lcnt.as<uint32_t>(),
                                              icc ? nullptr : ucnt.as<uint32_t>(),
                                              flags.as<unsigned>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  unsigned hf = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&hf, flags.ptr, sizeof(hf), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  require(!(hf & kUnsorted), VCLGB_INVALID_MATRIX,
          "Chow-Patel needs ascending, duplicate-free columns in every row");
  if (hf & kNoDiagonal) throw Error(VCLGB_ZERO_ON_DIAGONAL, "a row has no diagonal entry");
  if (hf & kZeroDiagonal) throw Error(VCLGB_ZERO_ON_DIAGONAL, "zero on diagonal");

  DevBuf lrp(((size_t)n + 1) * 4, be.stream), urp(((size_t)n + 1) * 4, be.stream);
  const uint64_t nl = extern_scan_u32(be, lcnt.as<uint32_t>(), n, lrp.as<uint32_t>());
  const uint64_t nu = icc ? 0 : extern_scan_u32(be, ucnt.as<uint32_t>(), n, urp.as<uint32_t>());
  DevBuf lci(std::max<uint64_t>(nl, 1) * 4, be.stream), lrow(std::max<uint64_t>(nl, 1) * 4, be.stream);
  DevBuf aL(std::max<uint64_t>(nl, 1) * vs, be.stream);
  DevBuf uci(std::max<uint64_t>(nu, 1) * 4, be.stream), uv(std::max<uint64_t>(nu, 1) * vs, be.stream);
  cp_split_kernel<T><<<g, 256, 0, be.stream>>>(
      n, A.row_ptr, A.col_idx, av, D.as<T>(), lrp.as<uint32_t>(), lci.as<uint32_t>(), aL.as<T>(),
      lrow.as<uint32_t>(), icc ? nullptr : urp.as<uint32_t>(), uci.as<uint32_t>(), uv.as<T>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  const int ge = waves_grid(be, 256, 8, nl + nu);
  // sweep state: values ping-pong between two copies (the reference's backups)
  DevBuf L0(std::max<uint64_t>(nl, 1) * vs, be.stream), L1(std::max<uint64_t>(nl, 1) * vs, be.stream);
  VCLGB_CUDA(cudaMemcpyAsync(L0.ptr, aL.ptr, nl * vs, cudaMemcpyDeviceToDevice, be.stream));
  DevBuf *Lcur = &L0, *Lnext = &L1;
  DevBuf U0, U1, utrp, utci, umap, utrow, aU;
  DevBuf *Ucur = &U0, *Unext = &U1;
  if (!icc) {
    // U^T: rows of the transpose ascending, as ilu_transpose (:430-500) builds them
    csr_transpose_pattern(be, n, n, nu, urp.as<uint32_t>(), uci.as<uint32_t>(), utrp, utci, umap);
    utrow.alloc(std::max<uint64_t>(nu, 1) * 4, be.stream);
    aU.alloc(std::max<uint64_t>(nu, 1) * vs, be.stream);
    U0.alloc(std::max<uint64_t>(nu, 1) * vs, be.stream);
    U1.alloc(std::max<uint64_t>(nu, 1) * vs, be.stream);
    cp_row_of_kernel<<<g, 256, 0, be.stream>>>(n, utrp.as<uint32_t>(), utrow.as<uint32_t>());
    const int gu = waves_grid(be, 256, 8, nu);
    cp_gather_kernel<T><<<gu, 256, 0, be.stream>>>(nu, umap.as<uint32_t>(), uv.as<T>(), aU.as<T>());
    be.launches += 2;
    VCLGB_CHECK_LAUNCH();
    VCLGB_CUDA(cudaMemcpyAsync(U0.ptr, aU.ptr, nu * vs, cudaMemcpyDeviceToDevice, be.stream));
  }
  for (uint32_t s = 0; s < P.sweeps; ++s) {
    if (icc)
      cp_icc_sweep_kernel<T><<<ge, 256, 0, be.stream>>>(
          n, nl, lrp.as<uint32_t>(), lci.as<uint32_t>(), lrow.as<uint32_t>(), aL.as<T>(),
          Lcur->as<T>(), Lnext->as<T>());
    else
      cp_ilu_sweep_kernel<T><<<ge, 256, 0, be.stream>>>(
          n, nl, nu, lrp.as<uint32_t>(), lci.as<uint32_t>(), lrow.as<uint32_t>(), aL.as<T>(),
          Lcur->as<T>(), Lnext->as<T>(), utrp.as<uint32_t>(), utci.as<uint32_t>(),
          utrow.as<uint32_t>(), aU.as<T>(), Ucur->as<T>(), Unext->as<T>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    std::swap(Lcur, Lnext);
    std::swap(Ucur, Unext);
  }

  // Neumann matrices and their diagonals
  P.cp_l = neumann_matrix(be, A.prec, n, nl);
  P.diag.alloc(std::max<size_t>(n, 1) * vs, be.stream);
  P.diag_u.alloc(std::max<size_t>(n, 1) * vs, be.stream);
  cp_neumann_kernel<T><<<g, 256, 0, be.stream>>>(
      n, lrp.as<uint32_t>(), lci.as<uint32_t>(), Lcur->as<T>(), true, P.diag.as<T>(),
      P.cp_l->own_row_ptr.as<uint32_t>(), P.cp_l->own_col_idx.as<uint32_t>(),
      P.cp_l->own_values.as<T>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  if (icc) {
    // U := L^T (ilu_transpose of the swept L), its diagonal first in every row
    DevBuf ltrp, ltci, lmap;
    csr_transpose_pattern(be, n, n, nl, lrp.as<uint32_t>(), lci.as<uint32_t>(), ltrp, ltci, lmap);
    DevBuf ltv(std::max<uint64_t>(nl, 1) * vs, be.stream);
    P.cp_u = neumann_matrix(be, A.prec, n, nl);
    cp_gather_kernel<T><<<ge, 256, 0, be.stream>>>(nl, lmap.as<uint32_t>(), Lcur->as<T>(),
                                                   ltv.as<T>());
    cp_neumann_kernel<T><<<g, 256, 0, be.stream>>>(
        n, ltrp.as<uint32_t>(), ltci.as<uint32_t>(), ltv.as<T>(), false, P.diag_u.as<T>(),
        P.cp_u->own_row_ptr.as<uint32_t>(), P.cp_u->own_col_idx.as<uint32_t>(),
        P.cp_u->own_values.as<T>());
    be.launches += 2;
    VCLGB_CHECK_LAUNCH();
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));  // ltrp/ltci/lmap/ltv freed after use
  } else {
    // U from U^T (ilu_transpose back: the same pattern as U, values moved by the map)
    P.cp_u = neumann_matrix(be, A.prec, n, nu);
    const int gu = waves_grid(be, 256, 8, nu);
    cp_scatter_kernel<T><<<gu, 256, 0, be.stream>>>(nu, umap.as<uint32_t>(), Ucur->as<T>(),
                                                    uv.as<T>());
    cp_neumann_kernel<T><<<g, 256, 0, be.stream>>>(
        n, urp.as<uint32_t>(), uci.as<uint32_t>(), uv.as<T>(), false, P.diag_u.as<T>(),
        P.cp_u->own_row_ptr.as<uint32_t>(), P.cp_u->own_col_idx.as<uint32_t>(),
        P.cp_u->own_values.as<T>());
    be.launches += 2;
    VCLGB_CHECK_LAUNCH();
  }
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));  // temporaries freed after use
  csr_analyse(be, *P.cp_l);
  csr_analyse(be, *P.cp_u);
  P.work.alloc((size_t)n * vs * 6, be.stream);
  T *w = P.work.as<T>();
  cp_recip_kernel<T><<<g, 256, 0, be.stream>>>(n, P.diag.as<T>(), P.diag_u.as<T>(), w + 4 * (size_t)n,
                                               w + 5 * (size_t)n);
  be.launches++;
  VCLGB_CHECK_LAUNCH();
}

std::unique_ptr<Precond> chow_patel_create(Backend &be, const Matrix &A, bool icc,
                                           uint32_t sweeps, uint32_t jacobi_iters) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT,
          "the Chow-Patel preconditioners are built from a compressed_matrix");
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "Chow-Patel needs a square matrix");
  auto P = std::make_unique<Precond>();
  P->kind = icc ? 4 : 3;
  P->prec = A.prec;
  P->rows = A.rows;
  P->sweeps = sweeps;
  P->jacobi_iters = jacobi_iters;
  if (A.prec == VCLGB_FLOAT64)
    cp_build<double>(be, A, icc, *P);
  else
    cp_build<float>(be, A, icc, *P);
  return P;
}

template <typename T>
static void cp_apply(Backend &be, const Precond &P, T *vec, const int *skip) {
  const size_t n = P.rows;
  if (n == 0) return;
  T *w = P.work.as<T>();
  T *bL = w, *bU = w + n, *x0 = w + 2 * n, *x1 = w + 3 * n;
  const T *rl = w + 4 * n, *ru = w + 5 * n;  // D_L^-1, D_U^-1
  const int g = waves_grid(be, 256, 8, n);
  const uint32_t J = P.jacobi_iters;
  Reduction red{nullptr, nullptr};
  if (J == 0) {  // x_L = D_L^-1 v; result = D_U^-1 x_L
    cp_scale_kernel<T, true><<<g, 256, 0, be.stream>>>(n, vec, rl, ru, vec, skip);
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    return;
  }
  cp_scale_kernel<T, false><<<g, 256, 0, be.stream>>>(n, vec, rl, nullptr, bL, skip);
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  // L phase: x_1 = N_L b_L + b_L, ..., the last step writes b_U = x_J D_U^-1
  const T *x = bL;
  for (uint32_t k = 0; k < J; ++k) {
    if (k + 1 == J) {
      spmv_launch<T>(be, *P.cp_l, x, 0, 1, EpiCpStep<T, true>{bU, bL, ru, skip}, red, bU, 0, 1,
                     T(1), T(0), skip);
    } else {
      T *out = k & 1 ? x1 : x0;
      spmv_launch<T>(be, *P.cp_l, x, 0, 1, EpiCpStep<T, false>{out, bL, nullptr, skip}, red, out,
                     0, 1, T(1), T(0), skip);
      x = out;
    }
  }
  // U phase from x = b_U; the last step writes the result into vec
  x = bU;
  for (uint32_t k = 0; k < J; ++k) {
    T *out = k + 1 == J ? vec : (k & 1 ? x1 : x0);
    spmv_launch<T>(be, *P.cp_u, x, 0, 1, EpiCpStep<T, false>{out, bU, nullptr, skip}, red, out, 0,
                   1, T(1), T(0), skip);
    x = out;
  }
}

void chow_patel_apply(Backend &be, const Precond &P, void *d_vec, const int *skip_flag) {
  if (P.prec == VCLGB_FLOAT64)
    cp_apply<double>(be, P, static_cast<double *>(d_vec), skip_flag);
  else
    cp_apply<float>(be, P, static_cast<float *>(d_vec), skip_flag);
}

}  // namespace vclgb
