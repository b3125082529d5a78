/*
 * vclgb.h -- C ABI of the GB300 sparse Krylov engine.
 *
 * The engine stands in for ViennaCL's CUDA backend on the sparse path.  Each
 * entry point below names the ViennaCL interface it replaces (paths relative
 * to the ViennaCL source tree).  The conventions follow libviennacl's C API
 * (libviennacl/include/viennacl.hpp): an opaque backend handle, a precision
 * enum, plain device pointers plus offset/stride for vectors, and a status
 * code in place of C++ exceptions.
 *
 * All pointers named d_* are device pointers on the backend's GPU.  Calls are
 * asynchronous on the backend's stream unless documented otherwise; solver
 * calls return after the solve has finished (they read back the iteration
 * count and residual estimate).  Everything is re-entrant across backends;
 * one backend must not be used from two host threads at once.
 */
#ifndef VCLGB_H
#define VCLGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define VCLGB_API __attribute__((visibility("default")))
#else
#define VCLGB_API
#endif

/* ---- status codes (libviennacl/include/viennacl.hpp:95-99 has only
 *      ViennaCLSuccess / ViennaCLGenericFailure; the codes are extended) ---- */
typedef enum {
  VCLGB_SUCCESS = 0,
  VCLGB_GENERIC_FAILURE = 1,
  VCLGB_INVALID_ARGUMENT = 2,
  VCLGB_INVALID_MATRIX = 3,     /* row_ptr not monotone, column out of range, ... */
  VCLGB_OUT_OF_MEMORY = 4,
  VCLGB_CUDA_ERROR = 5,
  VCLGB_NOT_CONVERGED = 6,      /* max iterations reached (result still written) */
  VCLGB_BREAKDOWN = 7,          /* NaN/Inf or zero divisor inside a solver */
  VCLGB_ZERO_ON_DIAGONAL = 8,   /* viennacl::zero_on_diagonal_exception (forwards.h:621) */
  VCLGB_TIMEOUT = 9,            /* a bounded device-side wait gave up */
  VCLGB_UNSUPPORTED = 10
} vclgbStatus;

/* ViennaCLPrecision (libviennacl/include/viennacl.hpp:75-80) */
typedef enum { VCLGB_FLOAT32 = 0, VCLGB_FLOAT64 = 1 } vclgbPrecision;

/* ---- backend: ViennaCLBackend (libviennacl/include/viennacl.hpp:104-113) -- */
typedef struct vclgbBackend_st *vclgbBackend;

/* Creates a backend on the current CUDA device using the given stream.
 * NULL: a blocking stream of the backend's own, ordered with the legacy
 * default stream as the reference's launches are, and destroyed with the
 * backend.  vclgbBackendSetStream moves the backend (and its scratch
 * buffers) to the caller's stream; a stream of the backend's own stays alive
 * until the backend is destroyed.  Matrices, preconditioners and batches
 * may be destroyed before or after their backend. */
VCLGB_API vclgbStatus vclgbBackendCreate(vclgbBackend *backend, void *cuda_stream);
VCLGB_API vclgbStatus vclgbBackendDestroy(vclgbBackend *backend);
VCLGB_API vclgbStatus vclgbBackendSetStream(vclgbBackend backend, void *cuda_stream);
VCLGB_API vclgbStatus vclgbBackendSynchronize(vclgbBackend backend);
/* Message of the last failure on this backend (never NULL). */
VCLGB_API const char *vclgbBackendLastError(vclgbBackend backend);
/* Number of kernel launches issued by this backend so far. */
VCLGB_API uint64_t vclgbBackendLaunchCount(vclgbBackend backend);
/* Library version string. */
VCLGB_API const char *vclgbVersion(void);

/* Kernel timing (a measurement hook with no reference counterpart; off by
 * default).  While enabled, every SpMV phase (kind 0: the product with its
 * fused epilogue, all formats) and every fused vector pass (kind 1) the
 * backend launches is bracketed by two CUDA events on its stream -- inside
 * the solvers' captured CUDA graphs as event nodes -- so that kernel
 * durations can be read from a real solve.  vclgbBackendKernelTimes copies up
 * to `capacity` durations in milliseconds (host array; may be NULL) of the
 * given kind recorded since the last call, sets *count to how many there
 * were, and clears them.  Enabling or disabling clears both lists. */
VCLGB_API vclgbStatus vclgbBackendSetKernelTiming(vclgbBackend be, int enable);
VCLGB_API vclgbStatus vclgbBackendKernelTimes(vclgbBackend be, int kind, float *h_ms,
                                              uint64_t capacity, uint64_t *count);

/* ---- sparse matrices ----------------------------------------------------- */
typedef struct vclgbMatrix_st *vclgbMatrix;

typedef enum {
  VCLGB_CSR = 0,   /* viennacl::compressed_matrix   (compressed_matrix.hpp:629-1198) */
  VCLGB_ELL = 1,   /* viennacl::ell_matrix          (ell_matrix.hpp:52-120) */
  VCLGB_SELL = 2,  /* viennacl::sliced_ell_matrix   (sliced_ell_matrix.hpp:45-133) */
  VCLGB_HYB = 3,   /* viennacl::hyb_matrix          (hyb_matrix.hpp:37-132) */
  VCLGB_COO = 4    /* viennacl::coordinate_matrix   (coordinate_matrix.hpp:186-397) */
} vclgbFormat;

/* compressed_matrix(row_ptr, cols, vals, CUDA_MEMORY, rows, cols, nnz): wraps
 * existing device arrays without copying (compressed_matrix.hpp:740-781).  The
 * caller keeps ownership and must keep them alive until the matrix is
 * destroyed.  Validates row_ptr/cols on the device (VCLGB_INVALID_MATRIX) and
 * runs the row-length analysis the adaptive CSR kernel uses. */
VCLGB_API vclgbStatus vclgbCsrCreate(vclgbBackend be, vclgbPrecision prec, uint32_t rows,
                                     uint32_t cols, uint32_t nnz, const uint32_t *d_row_ptr,
                                     const uint32_t *d_col_idx, const void *d_values,
                                     vclgbMatrix *out);

/* Format conversions, performed on the GPU from a CSR matrix; the result owns
 * its arrays.  Bit-identical to viennacl::copy(host_matrix, ...) of the same
 * rows with columns in CSR order:
 *   ELL : ell_matrix.hpp:123-171 (AlignmentV = 1)
 *   SELL: sliced_ell_matrix.hpp:140-214 for sigma = 1 (slice height C);
 *         sigma > 1 sorts rows by decreasing length in windows of sigma rows
 *         (stable) before slicing -- SELL-C-sigma, which the reference lacks
 *   HYB : hyb_matrix.hpp:135-234 with csr_threshold (ELL width = smallest k
 *         with at least threshold*rows rows of length <= k, compared in the
 *         matrix precision); the tail is kept both as the reference's CSR
 *         arrays and as COO for the segmented-reduction kernel. */
VCLGB_API vclgbStatus vclgbMatrixToEll(vclgbBackend be, vclgbMatrix csr, vclgbMatrix *out);
VCLGB_API vclgbStatus vclgbMatrixToSell(vclgbBackend be, vclgbMatrix csr, uint32_t slice_height,
                                        uint32_t sigma, vclgbMatrix *out);
VCLGB_API vclgbStatus vclgbMatrixToHyb(vclgbBackend be, vclgbMatrix csr, double csr_threshold,
                                       vclgbMatrix *out);
/* COO: viennacl::copy(host_matrix, coordinate_matrix<T, 128>)
 * (coordinate_matrix.hpp:46-101): (row, col) pairs interleaved in one u32
 * array and the values, both padded with zeros to a multiple of 128 entries,
 * plus the 65 group boundaries the reference computes (bit-identical,
 * including its rule that puts the first non-empty row alone in group 0 and
 * every later entry in group 63).  The product runs the warp-segmented
 * reduction over all entries and does not use the groups. */
VCLGB_API vclgbStatus vclgbMatrixToCoo(vclgbBackend be, vclgbMatrix csr, vclgbMatrix *out);
/* ell_matrix / sliced_ell_matrix / hyb_matrix that already live on the device
 * in the reference's layout (the CUDA buffers behind their handle() ...
 * handle5()), wrapped without copying; the arrays stay the caller's.
 *   ELL : ell_matrix<T, 1> (ell_matrix.hpp:52-120): coords/elems of rows*width
 *   SELL: sliced_ell_matrix<T, unsigned> (sliced_ell_matrix.hpp:45-133), sigma = 1
 *   HYB : hyb_matrix<T, 1> (hyb_matrix.hpp:37-132); tail_nnz = tail_row_ptr[rows]
 *         (the wrap derives the COO rows of the tail on the device). */
VCLGB_API vclgbStatus vclgbEllWrap(vclgbBackend be, vclgbPrecision prec, uint32_t rows,
                                   uint32_t cols, uint32_t width, const uint32_t *d_coords,
                                   const void *d_elems, vclgbMatrix *out);
VCLGB_API vclgbStatus vclgbSellWrap(vclgbBackend be, vclgbPrecision prec, uint32_t rows,
                                    uint32_t cols, uint32_t slice_height,
                                    const uint32_t *d_columns_per_block,
                                    const uint32_t *d_column_indices,
                                    const uint32_t *d_block_start, const void *d_elems,
                                    vclgbMatrix *out);
VCLGB_API vclgbStatus vclgbHybWrap(vclgbBackend be, vclgbPrecision prec, uint32_t rows,
                                   uint32_t cols, uint32_t ell_width,
                                   const uint32_t *d_ell_coords, const void *d_ell_elems,
                                   const uint32_t *d_tail_row_ptr, const uint32_t *d_tail_cols,
                                   const void *d_tail_vals, uint64_t tail_nnz, vclgbMatrix *out);
/* coordinate_matrix<T, A> already on the device (handle12() = interleaved
 * (row, col) pairs, handle() = values), entries sorted by row as the
 * reference's copy() leaves them; wrapped without copying.  d_coords must be
 * 8-byte aligned (the reference's CUDA kernel reads the pairs as uint2). */
VCLGB_API vclgbStatus vclgbCooWrap(vclgbBackend be, vclgbPrecision prec, uint32_t rows,
                                   uint32_t cols, uint64_t nnz, const uint32_t *d_coords,
                                   const void *d_elems, vclgbMatrix *out);
/* viennacl::io::read_matrix_market_file(matrix, path, index_base)
 * (io/matrix_market.hpp:101-369) straight into a device compressed_matrix that
 * owns its arrays.  Same file rules as the reference: "%%MatrixMarket matrix
 * coordinate real|complex|pattern general|symmetric" (complex keeps the real
 * part, pattern entries are 1), comment and blank lines, "rows cols nnz",
 * then nnz entries whose indices count from index_base (1 in the reference's
 * default); symmetric files set both A(i,j) and A(j,i); a later entry for the
 * same position replaces an earlier one.  *lines_read (may be NULL) receives
 * the reference's return value, the number of lines read.  A file that
 * cannot be opened, a bad header, index or number, or fewer entries than
 * announced returns VCLGB_INVALID_ARGUMENT with the cause (file, line) in
 * vclgbBackendLastError. */
VCLGB_API vclgbStatus vclgbReadMatrixMarket(vclgbBackend be, const char *path, int64_t index_base,
                                            vclgbPrecision prec, vclgbMatrix *out,
                                            uint64_t *lines_read);
/* viennacl::io::write_matrix_market_file(matrix, path, index_base)
 * (io/matrix_market.hpp:374-417) for a compressed_matrix: the "coordinate
 * real general" header, the size line, one entry per line in row order.
 * Values carry `digits` significant digits; 0 selects 6, the reference's
 * default stream precision (17 writes values that read back exactly). */
VCLGB_API vclgbStatus vclgbWriteMatrixMarket(vclgbBackend be, vclgbMatrix A, const char *path,
                                             int64_t index_base, int digits);
/* viennacl::reorder(matrix, cuthill_mckee_tag()) (misc/cuthill_mckee.hpp:366-421)
 * or, advanced != 0, reorder(matrix, advanced_cuthill_mckee_tag(a, gmax))
 * (misc/cuthill_mckee.hpp:429-605) on the pattern of a square CSR matrix, its
 * rows read in ascending column order as the reference's host maps hold them.
 * Writes d_perm[i] = new label of node i (rows device array), identical to
 * the reference's result.  The ordering itself is a sequential search and
 * runs on the host. */
VCLGB_API vclgbStatus vclgbCuthillMcKee(vclgbBackend be, vclgbMatrix A, int advanced,
                                        double starting_node_param, uint64_t max_root_nodes,
                                        uint32_t *d_perm);
/* B = P A P^T on the device: B(perm[i], perm[j]) = A(i, j), columns ascending
 * in every row of B; the result owns its arrays.  A perm that is not a
 * permutation of 0..rows-1 returns VCLGB_INVALID_ARGUMENT.  (The reference
 * leaves applying its permutation to the caller.) */
VCLGB_API vclgbStatus vclgbCsrPermute(vclgbBackend be, vclgbMatrix A, const uint32_t *d_perm,
                                      vclgbMatrix *out);
/* max over rows of (largest - smallest column index) -- the bandwidth measure
 * of misc/cuthill_mckee.hpp:46-76 for a fully numbered matrix. */
VCLGB_API vclgbStatus vclgbCsrBandwidth(vclgbBackend be, vclgbMatrix A, uint32_t *bandwidth);
/* FP32 copy of a matrix (same format and pattern), as mixed_precision_cg.hpp:128-137
 * builds for its inner iterations. */
VCLGB_API vclgbStatus vclgbMatrixToFloat32(vclgbBackend be, vclgbMatrix m, vclgbMatrix *out);
VCLGB_API vclgbStatus vclgbMatrixDestroy(vclgbMatrix *m);

/* Per-matrix SpMV autotuner (no reference counterpart; the reference's slice
 * height is the caller's and its CSR kernel a fixed rule,
 * linalg/cuda/sparse_matrix_operations.hpp:262-396).  Times the CSR kernel the
 * row-length analysis picks (lanes per row by length class) against
 * SELL-C-sigma for C in {32, 64} and sigma in {1, C, 256, 1024, 4096}, HYB
 * (csr_threshold 0.8) and ELL where it pads to at most twice the nonzeros,
 * each converted on the device and timed over ten products; forms padding
 * beyond 8 x nnz are skipped.  The fastest is kept with the matrix: from then
 * on vclgbSpmv and every solver's SpMV phase on `csr` run on it.  It is a
 * converted copy: after changing the matrix's values call
 * vclgbMatrixAutotuneClear (or tune again).  Host-synchronising. */
typedef struct {
  int32_t format;          /* chosen vclgbFormat (VCLGB_CSR: the CSR kernel won) */
  uint32_t slice_height;   /* SELL: C */
  uint32_t sigma;          /* SELL: sort window */
  uint32_t candidates;     /* forms tried, CSR included */
  double csr_threshold;    /* HYB: the threshold used */
  double us_csr;           /* microseconds per product, CSR kernel */
  double us_best;          /* microseconds per product, chosen form */
} vclgbTuneInfo;
VCLGB_API vclgbStatus vclgbMatrixAutotune(vclgbBackend be, vclgbMatrix csr, vclgbTuneInfo *info);
VCLGB_API vclgbStatus vclgbMatrixAutotuneClear(vclgbMatrix csr);

typedef struct {
  int32_t format;        /* vclgbFormat */
  int32_t precision;     /* vclgbPrecision */
  uint32_t rows, cols;
  uint64_t nnz;          /* nonzeros of the source pattern */
  uint64_t stored;       /* stored slots incl. padding (ELL/SELL/HYB-ELL part/COO) */
  uint32_t ell_width;    /* ELL: maxnnz; HYB: ellnnz */
  uint32_t slice_height; /* SELL: C */
  uint32_t sigma;        /* SELL: sort window */
  uint32_t num_slices;   /* SELL */
  uint64_t tail_nnz;     /* HYB: csr_nnz() incl. the one placeholder of an empty tail */
  uint32_t num_bins;     /* CSR: row-length bins of the adaptive kernel */
  uint32_t reserved;
} vclgbMatrixInfo;
VCLGB_API vclgbStatus vclgbMatrixGetInfo(vclgbMatrix m, vclgbMatrixInfo *info);

/* Copies one internal array into a caller-provided device buffer (sized from
 * vclgbMatrixGetInfo), for inspection and bit-exact parity checks:
 *   ELL : 0 coords u32[rows*width] (handle2), 1 elements T[rows*width] (handle)
 *   SELL: 0 columns_per_block u32[slices] (handle1), 1 column indices u32[stored]
 *         (handle2), 2 block_start u32[slices] (handle3), 3 elements T[stored]
 *         (handle), 4 row permutation u32[rows] (position -> row)
 *   HYB : 0 ell coords, 1 ell elements, 2 tail row_ptr u32[rows+1] (handle3),
 *         3 tail cols u32[tail_nnz] (handle4), 4 tail elements T[tail_nnz] (handle5)
 *   COO : 0 coords u32[2*stored] (handle12), 1 elements T[stored] (handle),
 *         2 group boundaries u32[65] (handle3); stored = nnz rounded up to 128
 *   CSR : 0 row_ptr, 1 cols, 2 values, 3 row blocks u32[nblocks+1] of
 *         generate_row_block_information (compressed_matrix.hpp:1152-1188);
 *         use vclgbCsrRowBlockCount for its length. */
VCLGB_API vclgbStatus vclgbMatrixExport(vclgbBackend be, vclgbMatrix m, int which, void *d_dst);
VCLGB_API vclgbStatus vclgbCsrRowBlockCount(vclgbBackend be, vclgbMatrix csr, uint32_t *count);

/* ---- SpMV: linalg::prod_impl(A, x, alpha, y, beta)
 *      (linalg/sparse_matrix_operations.hpp:90-121 -> linalg/cuda/sparse_matrix_operations.hpp
 *      prod_impl for compressed/ell/sliced_ell/hyb).  y = alpha*A*x + beta*y,
 *      y not read when beta == 0.  x/y are T arrays in the matrix precision;
 *      element i lives at start + i*stride.  x and y must not overlap. ---- */
VCLGB_API vclgbStatus vclgbSpmv(vclgbBackend be, vclgbMatrix A, double alpha, const void *d_x,
                                int64_t x_start, int64_t x_stride, double beta, void *d_y,
                                int64_t y_start, int64_t y_stride);

/* ---- vector reductions: inner_prod / norm_2 (linalg/inner_prod.hpp,
 *      linalg/norm_2.hpp -> cuda/vector_operations.hpp:1272-1585, 2017-2448).
 *      The result is written to a device scalar (d_result, same precision),
 *      with no host synchronisation. ---- */
VCLGB_API vclgbStatus vclgbDot(vclgbBackend be, vclgbPrecision prec, uint64_t n, const void *d_x,
                               int64_t x_start, int64_t x_stride, const void *d_y,
                               int64_t y_start, int64_t y_stride, void *d_result);
VCLGB_API vclgbStatus vclgbNorm2(vclgbBackend be, vclgbPrecision prec, uint64_t n,
                                 const void *d_x, int64_t x_start, int64_t x_stride,
                                 void *d_result);

/* ---- vector updates and element-wise operations (a vector is a device pointer
 *      of the given precision, element i at start + i*stride) ----------------- */
/* A scalar operand of av/avbv/element_op: a host value, or a device scalar of
 * the vectors' precision when d_value != NULL (viennacl::scalar<T>); negated
 * first when flip_sign != 0; divided by instead of multiplied with when
 * reciprocal != 0 (the len/reciprocal/flip_sign arguments of
 * linalg/vector_operations.hpp:78-183). */
typedef struct {
  double value;
  const void *d_value;
  int32_t reciprocal;
  int32_t flip_sign;
} vclgbScalarArg;

/* av / avbv / avbv_v (linalg/vector_operations.hpp:78-183; CUDA backend
 * linalg/cuda/vector_operations.hpp:77-760):
 *   d_z == NULL:  y = x op alpha           (av; accumulate != 0: y += x op alpha)
 *   otherwise:    y = x op alpha + z op beta   (avbv; accumulate != 0: y += ..., avbv_v)
 * with op * or / by the scalar's reciprocal flag.  Every product, quotient and
 * sum is rounded on its own (no fused multiply-add), so the result equals a
 * host evaluation of the same expression bit for bit.  y may alias x or z
 * element for element (same start and stride). */
VCLGB_API vclgbStatus vclgbAvbv(vclgbBackend be, vclgbPrecision prec, uint64_t n, void *d_y,
                                int64_t y_start, int64_t y_stride, const void *d_x,
                                int64_t x_start, int64_t x_stride, vclgbScalarArg alpha,
                                const void *d_z, int64_t z_start, int64_t z_stride,
                                vclgbScalarArg beta, int accumulate);

/* element_op with op_element_binary (linalg/vector_operations.hpp:255-345,
 * linalg/detail/op_applier.hpp): y = x OP z for OP element_prod (x*z),
 * element_div (x/z) or element_pow (pow(x, z)).  Either operand may be a
 * scalar instead: pass d_x == NULL (then x_scalar) or d_z == NULL (then
 * z_scalar); reciprocal is ignored there.  prod and div are correctly rounded
 * (bit-identical to the host); pow calls CUDA's pow. */
typedef enum { VCLGB_OP_PROD = 0, VCLGB_OP_DIV = 1, VCLGB_OP_POW = 2 } vclgbBinaryOp;
VCLGB_API vclgbStatus vclgbElementBinary(vclgbBackend be, vclgbPrecision prec, uint64_t n,
                                         void *d_y, int64_t y_start, int64_t y_stride,
                                         const void *d_x, int64_t x_start, int64_t x_stride,
                                         vclgbScalarArg x_scalar, const void *d_z,
                                         int64_t z_start, int64_t z_stride,
                                         vclgbScalarArg z_scalar, int op);

/* element_op with op_element_unary (linalg/detail/op_applier.hpp): y = f(x)
 * for the reference's unary functions; exp10 is exp(x ln 10) and rsqrt is
 * pow(x, -0.5), as the reference defines them.  The functions are CUDA's own
 * (results within its documented error bounds of the host's). */
typedef enum {
  VCLGB_OP_ABS = 16, VCLGB_OP_ACOS, VCLGB_OP_ACOSH, VCLGB_OP_ASIN, VCLGB_OP_ASINH,
  VCLGB_OP_ATAN, VCLGB_OP_ATANH, VCLGB_OP_CEIL, VCLGB_OP_COS, VCLGB_OP_COSH, VCLGB_OP_ERF,
  VCLGB_OP_ERFC, VCLGB_OP_EXP, VCLGB_OP_EXP2, VCLGB_OP_EXP10, VCLGB_OP_FABS, VCLGB_OP_FLOOR,
  VCLGB_OP_LOG, VCLGB_OP_LOG2, VCLGB_OP_LOG10, VCLGB_OP_ROUND, VCLGB_OP_SIN, VCLGB_OP_SINH,
  VCLGB_OP_SQRT, VCLGB_OP_TAN, VCLGB_OP_TANH, VCLGB_OP_TRUNC, VCLGB_OP_RSQRT, VCLGB_OP_SIGN
} vclgbUnaryOp;
VCLGB_API vclgbStatus vclgbElementUnary(vclgbBackend be, vclgbPrecision prec, uint64_t n,
                                        void *d_y, int64_t y_start, int64_t y_stride,
                                        const void *d_x, int64_t x_start, int64_t x_stride, int op);

/* vector_assign (linalg/vector_operations.hpp:187-216): y = alpha;
 * vector_swap (:218-250): exchanges x and y. */
VCLGB_API vclgbStatus vclgbVectorAssign(vclgbBackend be, vclgbPrecision prec, uint64_t n, void *d_y,
                                        int64_t y_start, int64_t y_stride, double alpha);
VCLGB_API vclgbStatus vclgbVectorSwap(vclgbBackend be, vclgbPrecision prec, uint64_t n, void *d_x,
                                      int64_t x_start, int64_t x_stride, void *d_y,
                                      int64_t y_start, int64_t y_stride);

/* ---- preconditioners -------------------------------------------------------- */
typedef struct vclgbPrecond_st *vclgbPrecond;

/* jacobi_precond<compressed_matrix>(A, jacobi_tag()) (linalg/jacobi_precond.hpp:103-130):
 * extracts diag(A) on the device (row_info SPARSE_ROW_DIAGONAL).  A zero
 * diagonal entry returns VCLGB_ZERO_ON_DIAGONAL. */
VCLGB_API vclgbStatus vclgbJacobiCreate(vclgbBackend be, vclgbMatrix A, vclgbPrecond *out);
/* row_scaling<compressed_matrix>(A, row_scaling_tag(norm)) (linalg/row_scaling.hpp:150-191):
 * a diagonal of row norms of A -- norm 0: max |a_ij|, 1: sum |a_ij|, 2: Euclidean
 * (row_info, linalg/host_based/sparse_matrix_operations.hpp:52-98) -- applied as
 * element_div like Jacobi.  Any other norm returns VCLGB_INVALID_ARGUMENT (the
 * reference throws unknown_norm_exception); a zero row is not checked, as in
 * the reference's compressed_matrix specialisation. */
VCLGB_API vclgbStatus vclgbRowScalingCreate(vclgbBackend be, vclgbMatrix A, uint32_t norm,
                                            vclgbPrecond *out);
/* ilu0_precond<compressed_matrix>(A, ilu0_tag(use_level_scheduling))
 * (linalg/detail/ilu/ilu0.hpp:189-352).  The factorisation runs on the
 * device, level-scheduled row by row; the level sets of L and U are built on
 * the device with the reference's elimination order (detail/ilu/common.hpp:50-187). */
VCLGB_API vclgbStatus vclgbIlu0Create(vclgbBackend be, vclgbMatrix A, int use_level_scheduling,
                                      vclgbPrecond *out);
/* block_ilu_precond<compressed_matrix, ilu0_tag>(A, ilu0_tag(), num_blocks) and the
 * block_boundaries constructor (linalg/detail/ilu/block_ilu.hpp:301-365): ILU0 of A
 * restricted to its diagonal blocks, factorised and applied on the device as
 * ilu0_precond is (vclgbIlu0GetInfo / vclgbIlu0Export work on it; the factors
 * lie in the block-diagonal pattern and equal the reference's per-block
 * factors).  h_bounds NULL: the reference's split [i*rows/num_blocks,
 * (i+1)*rows/num_blocks); else 2*num_blocks host values [start, stop) that must
 * tile [0, rows) (VCLGB_INVALID_ARGUMENT otherwise).  The reference's apply skips
 * the last column of U (its U^T row pointer ends at 0); this one applies it. */
VCLGB_API vclgbStatus vclgbBlockIlu0Create(vclgbBackend be, vclgbMatrix A, uint32_t num_blocks,
                                           const uint32_t *h_bounds, vclgbPrecond *out);
/* chow_patel_ilu_precond<compressed_matrix>(A, chow_patel_tag(sweeps, jacobi_iters))
 * and chow_patel_icc_precond (linalg/detail/ilu/chow_patel_ilu.hpp:44-70 tag,
 * :77-150 setup, :170-300 apply; reference defaults sweeps 3, jacobi_iters 2).
 * The setup runs on the device with the reference's operation order, so the
 * Neumann matrices I - D^-1 L, I - D^-1 U and the diagonals are bit-identical
 * to the host backend's.  A needs ascending, duplicate-free columns in every
 * row (else VCLGB_INVALID_MATRIX: the reference's merge assumes them) and a
 * nonzero diagonal entry in every row (else VCLGB_ZERO_ON_DIAGONAL, where the
 * reference asserts). */
VCLGB_API vclgbStatus vclgbChowPatelIluCreate(vclgbBackend be, vclgbMatrix A, uint32_t sweeps,
                                              uint32_t jacobi_iters, vclgbPrecond *out);
VCLGB_API vclgbStatus vclgbChowPatelIccCreate(vclgbBackend be, vclgbMatrix A, uint32_t sweeps,
                                              uint32_t jacobi_iters, vclgbPrecond *out);
typedef struct {
  uint32_t kind;                 /* 0 ILU, 1 ICC */
  uint32_t sweeps, jacobi_iters;
  uint64_t nnz_L, nnz_U;         /* strictly triangular entries of the Neumann matrices */
} vclgbChowPatelInfo;
VCLGB_API vclgbStatus vclgbChowPatelGetInfo(vclgbPrecond P, vclgbChowPatelInfo *info);
/* Exports, into device memory: 0 L row_ptr u32[rows+1], 1 L cols u32[nnz_L],
 * 2 L values T[nnz_L] (I - D_L^-1 L without its zero diagonal), 3 D_L T[rows],
 * 4..7 the same for U (ICC: L^T, and D_L again). */
VCLGB_API vclgbStatus vclgbChowPatelExport(vclgbBackend be, vclgbPrecond P, int which,
                                           void *d_dst);
/* precond.apply(vec) in place on a contiguous device vector of length rows. */
VCLGB_API vclgbStatus vclgbPrecondApply(vclgbBackend be, vclgbPrecond P, void *d_vec);
VCLGB_API vclgbStatus vclgbPrecondDestroy(vclgbPrecond *P);

typedef struct {
  uint32_t num_levels_L, num_levels_U;
  uint64_t rows_L, rows_U, nnz_L, nnz_U;
} vclgbIlu0Info;
VCLGB_API vclgbStatus vclgbIlu0GetInfo(vclgbPrecond P, vclgbIlu0Info *info);
/* Exports the ILU0 factors and level sets (flattened over levels):
 *   0 LU values T[nnz] (A's pattern, unit L implicit), 1 U diagonal T[rows],
 *   L: 2 level_ptr u32[levels+1], 3 row_index u32[rows_L], 4 row_ptr u32[rows_L+1],
 *      5 cols u32[nnz_L], 6 vals T[nnz_L];  U: 7..11 likewise (vals pre-divided
 *      by the row's U diagonal, as detail/ilu/common.hpp:162 does). */
VCLGB_API vclgbStatus vclgbIlu0Export(vclgbBackend be, vclgbPrecond P, int which, void *d_dst);

/* ---- triangular solves --------------------------------------------------------
 * inplace_solve(A, vec, tag) and, transposed != 0, inplace_solve(trans(A), vec, tag)
 * for a square compressed_matrix (host backend linalg/host_based/
 * sparse_matrix_operations.hpp:537-1090; CUDA backend linalg/cuda/
 * sparse_matrix_operations.hpp:780-1008).  tag: VCLGB_LOWER / VCLGB_UPPER divide by
 * the row's diagonal entry, VCLGB_UNIT_LOWER / VCLGB_UNIT_UPPER take a unit
 * diagonal; entries outside the tag's strict triangle are ignored, as in the
 * reference (a missing diagonal entry divides by zero there and here).  d_vec
 * is a contiguous device vector of length rows, overwritten by the solution.
 * The rows run level by level on the device; the levels depend on the
 * pattern only and are built on the first call for each (triangle,
 * orientation) and kept with the matrix, so the pattern must not change
 * afterwards (the values may). */
typedef enum { VCLGB_LOWER = 0, VCLGB_UPPER = 1, VCLGB_UNIT_LOWER = 2, VCLGB_UNIT_UPPER = 3 } vclgbTriTag;
VCLGB_API vclgbStatus vclgbCsrInplaceSolve(vclgbBackend be, vclgbMatrix A, int tag, int transposed,
                                           void *d_vec);

/* ---- iterative solvers ------------------------------------------------------ */
/* Mirrors cg_tag / bicgstab_tag / gmres_tag (linalg/cg.hpp:48-87,
 * linalg/bicgstab.hpp:47-90, linalg/gmres.hpp:49-101); iters and error are
 * outputs, like the tags' mutable members. */
typedef struct {
  double tol;                       /* relative tolerance */
  double abs_tol;                   /* absolute tolerance (default 0) */
  uint32_t max_iters;
  uint32_t krylov_dim;              /* GMRES restart length */
  uint32_t max_iters_before_restart;/* BiCGStab (generic preconditioned variant) */
  uint32_t check_every;             /* iterations a trip of the device-side loop
                                       runs before its status test (0 = automatic) */
  /* outputs */
  uint32_t iters;
  uint32_t status;                  /* vclgbStatus of the solve */
  double error;                     /* the solver's own relative residual estimate */
} vclgbSolverTag;

/* Fills a tag with the reference defaults of the given solver kind
 * (0 = cg: 1e-8/300, 1 = bicgstab: 1e-8/400/200, 2 = gmres: 1e-10/300/20). */
VCLGB_API void vclgbSolverTagInit(vclgbSolverTag *tag, int kind);

/* linalg::solve(A, b, cg_tag[, precond]).  precond == NULL runs the pipelined
 * Chronopoulos-Gear CG (linalg/cg.hpp:128-187), otherwise the preconditioned
 * CG of linalg/cg.hpp:257-322, with the same stopping tests.  The whole
 * iteration (SpMV, reductions, scalar recurrences, convergence test) runs on
 * the device, looping in a CUDA graph until the status word says done; the
 * host waits once.  Systems of up to 32,768 rows (CSR, no preconditioner or a
 * diagonal one; at most 2,048 rows a CTA of the cluster) run in one
 * thread-block-cluster launch.  Large stencil-like systems (one row-length
 * bin, vectors of 32 MB or more, vectors and matrix beyond L2) keep their
 * vectors in a persisting L2 window: for the duration of the call the
 * current context's cudaLimitPersistingL2CacheSize is raised, and it is back
 * at the caller's value when the call returns (overlapping calls in the
 * process share one set-aside; the last to return restores it).
 * d_b, d_x: contiguous device vectors of length rows; x is overwritten
 * (initial guess 0, as in the reference). */
VCLGB_API vclgbStatus vclgbSolveCG(vclgbBackend be, vclgbMatrix A, const void *d_b, void *d_x,
                                   vclgbSolverTag *tag, vclgbPrecond precond);
/* linalg::solve(A, b, bicgstab_tag[, precond]): pipelined (bicgstab.hpp:96-215)
 * without, generic (bicgstab.hpp:398-489) with a preconditioner.  Systems of
 * up to 32,768 rows (CSR, no preconditioner or a diagonal one; at most 2,048
 * rows a CTA of the cluster) run in one thread-block-cluster launch.  Large
 * stencil-like systems use the persisting L2 window described for
 * vclgbSolveCG. */
VCLGB_API vclgbStatus vclgbSolveBiCGStab(vclgbBackend be, vclgbMatrix A, const void *d_b,
                                         void *d_x, vclgbSolverTag *tag, vclgbPrecond precond);
/* linalg::solve(A, b, gmres_tag[, precond]).  precond == NULL runs the
 * pipelined "simpler GMRES" with classical Gram-Schmidt (gmres.hpp:181-367);
 * with a preconditioner (any of the objects above) it follows the reference's
 * Householder variant (gmres.hpp:449-631): r = M^-1 (b - A x) and the
 * restart test rho_0/||b|| < tol, one iteration per Krylov step, the clamped
 * projection and the test |rho rho_0/||b||| < tol after every step.  Its
 * orthonormal basis is formed by classical Gram-Schmidt with one repeated
 * pass when the first cancelled more than half of the vector's norm squared
 * (the same basis as the reflections', up to rounding).  The restart
 * bookkeeping (triangular solve of size krylov_dim) runs on the device too.
 * Without a preconditioner, small CSR systems (krylov_dim <= 32, x, r and
 * the basis within the cluster's shared memory: up to 8,192 rows in FP64 at
 * krylov_dim 30, 16,384 at 20) run in one thread-block-cluster launch. */
VCLGB_API vclgbStatus vclgbSolveGMRES(vclgbBackend be, vclgbMatrix A, const void *d_b, void *d_x,
                                      vclgbSolverTag *tag, vclgbPrecond precond);
/* linalg::solve(A, b, mixed_precision_cg_tag(tol, max_iters, inner_tol))
 * (mixed_precision_cg.hpp:99-186): FP32 CG restarted from an FP64 residual. */
VCLGB_API vclgbStatus vclgbSolveMixedCG(vclgbBackend be, vclgbMatrix A, const void *d_b,
                                        void *d_x, vclgbSolverTag *tag, float inner_tol);

/* FP64 iterative refinement around FP32 Jacobi-PCG inner solves (no reference
 * counterpart).  FP64 is used only for r = b - A x, x += d and ||r||; the
 * inner solves run on an FP32 copy of A (built once and cached on A) to the
 * relative tolerance inner_tol (tightened no further than the outer target
 * needs).  tag->iters = total inner iterations; outer_iters (optional) gets
 * the number of refinement steps; tag->error = true FP64 ||b-Ax||/||b||. */
VCLGB_API vclgbStatus vclgbSolveRefinedCG(vclgbBackend be, vclgbMatrix A, const void *d_b,
                                          void *d_x, vclgbSolverTag *tag, double inner_tol,
                                          uint32_t max_outer, uint32_t *outer_iters);

/* ---- batched solves (no reference counterpart) ----------------------------
 * Many independent systems, given as the diagonal blocks of one FP64
 * block-diagonal CSR matrix A: system k owns rows [sys_ptr[k], sys_ptr[k+1])
 * and every entry of those rows lies in the same column range (checked:
 * VCLGB_INVALID_MATRIX otherwise).  method[k] = 0 runs the pipelined CG of
 * cg.hpp:128-187, 1 the pipelined BiCGStab of bicgstab.hpp:96-215, each with
 * the reference's stopping test.  One persistent launch solves the batch:
 * CTAs pull whole systems from a device work queue, largest first, and each
 * system stops on its own convergence test.  The batch keeps a pointer to A
 * (destroy the batch first).  h_* arrays are host arrays of num_systems. */
typedef struct vclgbBatch_st *vclgbBatch;
VCLGB_API vclgbStatus vclgbBatchCreate(vclgbBackend be, vclgbMatrix A, uint32_t num_systems,
                                       const uint32_t *h_sys_ptr, const int32_t *h_methods,
                                       vclgbBatch *out);
/* Autotunes block size (128/256/512) and lanes per row (1/2/4/8) on every
 * eighth system; block/lanes (optional) receive the choice. */
VCLGB_API vclgbStatus vclgbBatchTune(vclgbBackend be, vclgbBatch batch, const void *d_b,
                                     int32_t *block, int32_t *lanes);
/* Solves all systems to relative tolerance tol (x overwritten, initial guess
 * 0).  Per-system iterations, status (vclgbStatus) and residual estimate are
 * written to the optional host arrays.  Returns VCLGB_SUCCESS when every
 * system converged, VCLGB_NOT_CONVERGED otherwise. */
VCLGB_API vclgbStatus vclgbBatchSolve(vclgbBackend be, vclgbBatch batch, const void *d_b,
                                      void *d_x, double tol, uint32_t max_iters,
                                      uint32_t *h_iters, int32_t *h_status, double *h_error);
VCLGB_API vclgbStatus vclgbBatchDestroy(vclgbBatch *batch);

/* ---- adjoint (backward) solve (no reference counterpart) ------------------
 * For x = A^-1 b (the forward solve) and dL/dx: solves A^T lambda = dL/dx with
 * solver 0 = CG, 1 = BiCGStab, 2 = GMRES (tag as for the forward solvers;
 * precond: NULL or a Jacobi preconditioner of A, which is also one of A^T;
 * GMRES with Jacobi runs the preconditioned variant of vclgbSolveGMRES),
 * writes dL/db = lambda (length rows) and, if d_dLdA != NULL, the gradient
 * on the sparsity pattern dL/dA_ij = -lambda_i x_j (length nnz, in A's entry
 * order).  symmetric != 0 uses A itself; otherwise A^T is built once on the
 * device with a map to A's entries and cached on A. */
VCLGB_API vclgbStatus vclgbSolveAdjoint(vclgbBackend be, vclgbMatrix A, int solver,
                                        vclgbPrecond precond, const void *d_x,
                                        const void *d_dLdx, void *d_dLdb, void *d_dLdA,
                                        vclgbSolverTag *tag, int symmetric);
/* The cached transpose of A (built on first use): 0 row_ptr u32[cols+1],
 * 1 cols u32[nnz], 2 values T[nnz], 3 map u32[nnz] (A entry of each A^T entry). */
VCLGB_API vclgbStatus vclgbTransposeExport(vclgbBackend be, vclgbMatrix A, int which,
                                           void *d_dst);

/* ---- HYB SpMV without allocation (no counterpart in the reference) --------
 * For callers that may not allocate device memory at call time: plug-ins
 * whose host application owns every device allocation through its own
 * allocator, services that reserve their whole memory budget at start-up,
 * and latency-bound loops that cannot take the synchronisation an
 * allocation may cause.  The regular HYB product (vclgbSpmv) allocates a small
 * carry buffer per call and the engine's matrix objects allocate when built;
 * this entry point allocates nothing and needs no backend.
 *
 * y = alpha*A*x + beta*y for A given directly as the hyb_matrix arrays of the
 * reference (hyb_matrix.hpp: handle2/handle = ELL coords/values of
 * rows*ell_width slots, column-major; handle3/4/5 = tail row_ptr[rows+1],
 * cols, values).  tail_nnz = tail_row_ptr[rows] (0 for an empty tail, whose
 * arrays hold one placeholder entry).  x and y are contiguous, x has the
 * matrix's column count, y has rows entries; the call is asynchronous on
 * cuda_stream (NULL = legacy default stream).
 *
 * The tail's segmented reduction keeps its carries in one fixed device array
 * inside the library, sized for tail_nnz <= 8,388,608 (768 KiB, held on
 * every GPU that loads the library until the process exits); a larger tail
 * returns VCLGB_INVALID_ARGUMENT before anything is launched.  The first call
 * on a device looks up that array's device address with the device current
 * (a one-time set-up); make the first call before any stream capture.  All
 * calls on a device share the array and it keeps the last call's contents:
 * calls that overlap on the GPU (different streams at the same time) race.
 * A CUDA error already pending on the calling thread when the call begins is
 * left in place for its owner (not cleared): the call then launches nothing
 * and returns VCLGB_CUDA_ERROR; an error of this call's own launches returns
 * VCLGB_CUDA_ERROR too. */
VCLGB_API vclgbStatus vclgbHybSpmvNoAlloc(void *cuda_stream, vclgbPrecision prec, uint32_t rows,
                                          uint32_t ell_width, const uint32_t *d_ell_coords,
                                          const void *d_ell_elems, const uint32_t *d_tail_row_ptr,
                                          const uint32_t *d_tail_cols, const void *d_tail_vals,
                                          uint64_t tail_nnz, double alpha, const void *d_x,
                                          double beta, void *d_y);

#ifdef __cplusplus
}
#endif
#endif /* VCLGB_H */
