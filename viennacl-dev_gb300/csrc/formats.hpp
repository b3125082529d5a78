// formats.hpp -- declarations shared between the engine's translation units.
#pragma once

#include "vclgb_internal.hpp"

namespace vclgb {

std::unique_ptr<Matrix> convert_ell(Backend &be, const Matrix &csr);
std::unique_ptr<Matrix> convert_sell(Backend &be, const Matrix &csr, uint32_t C, uint32_t sigma);
void sell_wide_chunks(Backend &be, Matrix &m);
std::unique_ptr<Matrix> convert_hyb(Backend &be, const Matrix &csr, double threshold);
std::unique_ptr<Matrix> convert_f32(Backend &be, const Matrix &m);
std::unique_ptr<Matrix> convert_coo(Backend &be, const Matrix &csr);
// DIA form of a CSR matrix whose entries lie on at most kMaxDiag diagonals
// and whose diagonals hold at most max_fill times its nonzeros; else null
std::unique_ptr<Matrix> try_convert_dia(Backend &be, const Matrix &csr, double max_fill);
// COO wrapped from reference arrays: checks the pairs, then derives the groups
void coo_validate(Backend &be, const Matrix &m);
void coo_groups(Backend &be, Matrix &m);
// COO row of every tail entry from the tail row_ptr (HYB wrapped from reference arrays)
void tail_rows_from_rp(Backend &be, uint32_t rows, const uint32_t *trp, uint64_t tnnz,
                       uint32_t *trow);
void csr_row_blocks(Backend &be, Matrix &m);
// out[0..n) = exclusive scan of in, out[n] = total; returns the total (host-synchronising)
uint64_t extern_scan_u32(Backend &be, const uint32_t *in, size_t n, uint32_t *out);

// MatrixMarket files (mmio.cu)
std::unique_ptr<Matrix> read_matrix_market(Backend &be, const char *path, long index_base,
                                           vclgbPrecision prec, uint64_t *lines_read);
void write_matrix_market(Backend &be, const Matrix &m, const char *path, long index_base,
                         int digits);

// bandwidth reduction (reorder.cu)
void cuthill_mckee_perm(Backend &be, const Matrix &A, bool advanced, double a, uint64_t gmax,
                        uint32_t *d_perm);
std::unique_ptr<Matrix> csr_permute(Backend &be, const Matrix &A, const uint32_t *d_perm);
uint32_t csr_bandwidth(Backend &be, const Matrix &A);

// transpose of a CSR pattern: rows of the transpose list their source rows in
// ascending order; map[k] = position in (rp, ci) of transposed entry k (adjoint.cu)
void csr_transpose_pattern(Backend &be, uint32_t rows, uint32_t cols, uint64_t nnz,
                           const uint32_t *rp, const uint32_t *ci, DevBuf &trp, DevBuf &tci,
                           DevBuf &map);

// preconditioners (precond.cu, chow_patel.cu)
std::unique_ptr<Precond> jacobi_create(Backend &be, const Matrix &A);
std::unique_ptr<Precond> row_scaling_create(Backend &be, const Matrix &A, uint32_t norm);
std::unique_ptr<Precond> ilu0_create(Backend &be, const Matrix &A, bool level_scheduling);
std::unique_ptr<Precond> block_ilu0_create(Backend &be, const Matrix &A, uint32_t num_blocks,
                                           const uint32_t *h_bounds);
std::unique_ptr<Precond> chow_patel_create(Backend &be, const Matrix &A, bool icc,
                                           uint32_t sweeps, uint32_t jacobi_iters);
void chow_patel_apply(Backend &be, const Precond &P, void *d_vec, const int *skip_flag);
// inplace_solve(A or trans(A), vec, tag) for a square CSR matrix; tag 0 lower,
// 1 upper, 2 unit_lower, 3 unit_upper (precond.cu)
void csr_inplace_solve(Backend &be, Matrix &A, int tag, bool trans, void *d_vec);
// z = M^-1 z in place; skipped on the device when *skip_flag != 0
void precond_apply(Backend &be, const Precond &P, void *d_vec, const int *skip_flag);
// diag(A) into a device buffer of the matrix precision; returns 1 in *zero_found
// if a diagonal entry is zero (host-synchronising)
void extract_diag(Backend &be, const Matrix &A, DevBuf &out, bool check_zero);

// per-matrix SpMV autotuner (tune.cu): keeps the fastest form on A (A.tuned)
void matrix_autotune(Backend &be, Matrix &A, vclgbTuneInfo *info);

// a strided vector operand: element i at p[start + i * stride]
struct VecArg {
  const void *p;
  int64_t start, stride;
};
// vector updates and element-wise operations (blas1.cu)
void avbv(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y, const VecArg &x,
          const vclgbScalarArg &a, const VecArg *z, const vclgbScalarArg *b, bool accumulate);
void element_binary(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y,
                    const VecArg *x, const vclgbScalarArg &xs, const VecArg *z,
                    const vclgbScalarArg &zs, int op);
void element_unary(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y,
                   const VecArg &x, int op);
void vector_assign(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &y, double a);
void vector_swap(Backend &be, vclgbPrecision prec, uint64_t n, const VecArg &x, const VecArg &y);

// vector reductions (blas1.cu)
void dot_launch(Backend &be, vclgbPrecision prec, uint64_t n, const void *x, int64_t xs,
                int64_t xinc, const void *y, int64_t ys, int64_t yinc, void *d_result,
                bool sqrt_result);

}  // namespace vclgb
