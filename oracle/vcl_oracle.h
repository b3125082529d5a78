/*
 * vcl_oracle.h -- CPU restatement of ViennaCL's host (OpenMP) backend for the
 * sparse Krylov path.  TEST INFRASTRUCTURE ONLY: this library is the checker
 * that the GPU engine is compared against (and the timed CPU baseline); the
 * product never links, loads or calls it.
 *
 * Every function names the reference file:line whose behaviour it restates.
 * Index type is 32-bit unsigned, as in the reference (unsigned int row_ptr/cols).
 */
#ifndef VCL_ORACLE_H
#define VCL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef uint32_t vo_u32;

/* ---- threads -------------------------------------------------------- */
int  vo_max_threads(void);
void vo_set_threads(int n);

/* ---- CSR SpMV: y = alpha*A*x + beta*y  (beta==0: y not read) -------- */
void vo_csr_spmv_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                   const double *x, double alpha, double beta, double *y);
void vo_csr_spmv_s(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const float *v,
                   const float *x, float alpha, float beta, float *y);
/* strided variant: x[col*xinc + xstart], y[row*yinc + ystart] */
void vo_csr_spmv_strided_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                           const double *x, size_t xstart, size_t xinc, double alpha,
                           double beta, double *y, size_t ystart, size_t yinc);

/* diagonal extraction (row_info SPARSE_ROW_DIAGONAL) */
void vo_csr_diag_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, double *d);
void vo_csr_diag_s(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const float *v, float *d);
void vo_row_norms_d(vo_u32 n, const vo_u32 *rp, const double *v, vo_u32 norm, double *d);

/* CSR-adaptive row blocks (compressed_matrix::generate_row_block_information).
 * blocks must hold n+1 entries; returns the number of blocks. */
size_t vo_csr_row_blocks(vo_u32 n, const vo_u32 *rp, vo_u32 *blocks);

/* ---- ELL ------------------------------------------------------------ */
vo_u32 vo_ell_width(vo_u32 n, const vo_u32 *rp);
/* coords/elems hold n*width entries (column-major: item*n + row), zero padded */
void vo_ell_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                   vo_u32 width, vo_u32 *coords, double *elems);
void vo_ell_spmv_d(vo_u32 n, vo_u32 width, const vo_u32 *coords, const double *elems,
                   const double *x, double alpha, double beta, double *y);

/* ---- SELL-C-sigma ---------------------------------------------------- */
/* perm[i] = original row stored at position i (identity for sigma == 1).
 * nslices = (n-1)/C + 1.  Fills columns_per_block[nslices], block_start[nslices]
 * and returns the total number of stored slots. */
size_t vo_sell_layout(vo_u32 n, const vo_u32 *rp, vo_u32 C, vo_u32 sigma,
                      vo_u32 *perm, vo_u32 *columns_per_block, vo_u32 *block_start);
void vo_sell_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, vo_u32 C,
                    const vo_u32 *perm, const vo_u32 *columns_per_block,
                    const vo_u32 *block_start, vo_u32 *coords, double *elems);
void vo_sell_spmv_d(vo_u32 n, vo_u32 C, const vo_u32 *perm, const vo_u32 *columns_per_block,
                    const vo_u32 *block_start, const vo_u32 *coords, const double *elems,
                    const double *x, double alpha, double beta, double *y);

/* ---- HYB ------------------------------------------------------------ */
/* ELL width chosen by the threshold rule evaluated in the value precision
 * (is_float selects float arithmetic for the comparison). Returns width and
 * the CSR-tail nnz (without the single placeholder entry for an empty tail). */
vo_u32 vo_hyb_width(vo_u32 n, vo_u32 ncols, const vo_u32 *rp, double threshold, int is_float,
                    size_t *tail_nnz);
void vo_hyb_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, vo_u32 width,
                   vo_u32 *ell_coords, double *ell_elems, vo_u32 *tail_rp, vo_u32 *tail_ci,
                   double *tail_v);
void vo_hyb_spmv_d(vo_u32 n, vo_u32 width, const vo_u32 *ell_coords, const double *ell_elems,
                   const vo_u32 *tail_rp, const vo_u32 *tail_ci, const double *tail_v,
                   const double *x, double alpha, double beta, double *y);
size_t vo_coo_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                     vo_u32 *coords, double *elems, vo_u32 *groups);
void vo_coo_spmv_d(vo_u32 n, size_t nnz, const vo_u32 *coords, const double *elems,
                   const double *x, double alpha, double beta, double *y);

/* ---- solvers ---------------------------------------------------------- */
typedef struct {
  double   tol;
  double   abs_tol;
  vo_u32   max_iters;
  vo_u32   krylov_dim;          /* GMRES */
  vo_u32   max_iters_before_restart; /* BiCGStab */
  vo_u32   iters;               /* out */
  double   error;               /* out: the solver's own estimate */
} vo_tag;

enum { VO_PRECOND_NONE = 0, VO_PRECOND_JACOBI = 1, VO_PRECOND_ILU0 = 2, VO_PRECOND_CHOW_PATEL = 3,
       VO_PRECOND_BLOCK_ILU0 = 4 };

typedef struct {
  int            kind;
  const double  *diag;        /* Jacobi: diag(A); Chow-Patel: D_L */
  /* ILU0: factors stored in A's pattern (unit L implicit), plus U diagonal */
  const vo_u32  *rp;
  const vo_u32  *ci;
  const double  *lu;
  const double  *udiag;       /* ILU0: U diagonal; Chow-Patel: D_U */
  /* Chow-Patel: the Neumann matrices I - D_L^-1 L and I - D_U^-1 U in CSR
   * (their diagonal entries stored as zeros, as the reference keeps them) */
  const vo_u32  *l_rp, *l_ci;
  const double  *l_v;
  const vo_u32  *u_rp, *u_ci;
  const double  *u_v;
  vo_u32         jacobi_iters;
} vo_precond;

void vo_precond_apply_d(vo_u32 n, const vo_precond *P, double *vec);

/* CG: kind NONE runs the pipelined (Chronopoulos-Gear) variant, any other kind
 * the generic preconditioned variant, exactly as the reference dispatches. */
void vo_cg_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
             double *x, vo_tag *tag, const vo_precond *P);
void vo_bicgstab_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
                   double *x, vo_tag *tag, const vo_precond *P);
/* GMRES: kind NONE runs the pipelined variant, any other kind the Householder
 * variant of gmres.hpp:449-631, as the reference dispatches. */
void vo_gmres_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
                double *x, vo_tag *tag, const vo_precond *P);
/* 1: the Householder GMRES ends a cycle at a clamp of xi without declaring
 * convergence and lets the next restart's true residual decide (the engine's
 * rule); 0 (default): the reference's rho = 0 verdict */
void vo_set_gmres_clamp_restart(int on);
/* pins the GMRES restatement to the host backend's stage-1 partition */
void vo_set_gmres_host_quirk(int on);
/* mixed_precision_cg (FP32 inner CG, FP64 restarts), inner_tol as in the tag */
void vo_mixed_cg_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
                   double *x, vo_tag *tag, float inner_tol);
/* FP64 iterative refinement around FP32 Jacobi-PCG inner solves. */
void vo_ir_jacobi_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                    const double *b, double *x, double tol, vo_u32 max_outer, double inner_tol,
                    vo_u32 max_inner, vo_u32 *outer_out, vo_u32 *inner_total_out,
                    double *relres_out);

/* ---- CSR triangular solves (inplace_solve) ------------------------------ */
/* tag 0 lower, 1 upper, 2 unit_lower, 3 unit_upper; trans != 0 solves with A^T */
void vo_csr_inplace_solve_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                            double *vec, int tag, int trans);

/* ---- ILU0 --------------------------------------------------------------- */
/* lu holds a copy of v on entry and the ILU0 factors on exit. */
void vo_ilu0_factor_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, double *lu);
/* Level-schedule setup (lower: setup_U = 0, upper: 1), flattened over levels:
 *   level_ptr[nlev+1]       offsets of each level's rows in row_index
 *   row_index[total_rows]   the row each level entry updates (ascending in a level)
 *   row_ptr[total_rows+1]   global CSR offsets into cols/vals
 *   cols/vals[total_nnz]    (upper: vals pre-divided by the row's U diagonal)
 * Call once with NULL arrays to get nlev (return), total_rows and total_nnz. */
size_t vo_level_setup_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *lu,
                        const double *udiag, int setup_U, size_t *total_rows, size_t *total_nnz,
                        vo_u32 *level_ptr, vo_u32 *row_index, vo_u32 *row_ptr, vo_u32 *cols,
                        double *vals);
/* one triangle's level-scheduled substitution */
void vo_level_substitute_d(size_t nlev, const vo_u32 *level_ptr, const vo_u32 *row_index,
                           const vo_u32 *row_ptr, const vo_u32 *cols, const double *vals,
                           double *vec);

/* ---- block ILU0 ---------------------------------------------------------- */
/* block_ilu_precond<compressed_matrix, ilu0_tag>::apply: rp/ci/lu hold the
 * ILU0 factors of A's block-diagonal part (columns ascending in every row). */
void vo_block_ilu0_apply_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *lu,
                           double *vec);
/* 1: skip U's last column as the reference's apply does (pinning only) */
void vo_set_block_ilu_host_quirk(int on);

/* ---- Chow-Patel ILU / ICC ----------------------------------------------- */
/* Entries of A with col <= row (L) and col >= row (U). */
void vo_cp_counts(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, size_t *nnz_l, size_t *nnz_u);
/* chow_patel_ilu_precond setup: L (lower incl. diagonal, A's order) and U
 * (upper incl. diagonal) as Neumann matrices with their diagonals D_L, D_U. */
void vo_chow_patel_ilu_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                         vo_u32 sweeps, vo_u32 *l_rp, vo_u32 *l_ci, double *l_v, double *diag_l,
                         vo_u32 *u_rp, vo_u32 *u_ci, double *u_v, double *diag_u);
/* chow_patel_icc_precond setup: L and its transpose as Neumann matrices, D_L. */
void vo_chow_patel_icc_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                         vo_u32 sweeps, vo_u32 *l_rp, vo_u32 *l_ci, double *l_v,
                         vo_u32 *lt_rp, vo_u32 *lt_ci, double *lt_v, double *diag_l);

/* ---- dense vector helpers ------------------------------------------------ */
double vo_dot_d(size_t n, const double *a, const double *b);
double vo_rel_residual_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                         const double *x, const double *b);

/* ---- CSR transpose (adjoint path) --------------------------------------- */
/* Builds A^T in CSR (columns sorted) and map[k_t] = position of that entry in A. */
void vo_csr_transpose_d(vo_u32 n_rows, vo_u32 n_cols, const vo_u32 *rp, const vo_u32 *ci,
                        const double *v, vo_u32 *trp, vo_u32 *tci, double *tv, vo_u32 *map);

#ifdef __cplusplus
}
#endif
#endif
