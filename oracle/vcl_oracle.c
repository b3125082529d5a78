/*
 * vcl_oracle.c -- CPU restatement of ViennaCL's host/OpenMP backend for the
 * sparse Krylov path.  TEST INFRASTRUCTURE ONLY (the checker and the timed CPU
 * baseline); the GPU engine never links or calls this file.
 *
 * Reference paths below are relative to the ViennaCL source tree.
 * Compiled with -ffp-contract=off so x86 and Arm builds round identically.
 */
#include "vcl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int vo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void vo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* OpenMP is used only above this size, as VIENNACL_OPENMP_VECTOR_MIN_SIZE does
 * (viennacl/linalg/host_based/common.hpp). */
#define VO_OMP_MIN 5000

/* ------------------------------------------------------------------------ */
/* CSR SpMV -- host_based/sparse_matrix_operations.hpp:153-186              */
/* ------------------------------------------------------------------------ */
#define VO_DEF_CSR_SPMV(T, S)                                                          \
  void vo_csr_spmv_##S(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const T *v,        \
                       const T *x, T alpha, T beta, T *y) {                              \
    long r;                                                                             \
    _Pragma("omp parallel for if(n > VO_OMP_MIN)")                                      \
    for (r = 0; r < (long)n; ++r) {                                                     \
      T acc = 0;                                                                        \
      vo_u32 k, e = rp[r + 1];                                                          \
      for (k = rp[r]; k < e; ++k) acc += v[k] * x[ci[k]];                               \
      if (beta < 0 || beta > 0)                                                         \
        y[r] = alpha * acc + beta * y[r];                                               \
      else                                                                              \
        y[r] = alpha * acc;                                                             \
    }                                                                                   \
  }
VO_DEF_CSR_SPMV(double, d)
VO_DEF_CSR_SPMV(float, s)

void vo_csr_spmv_strided_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                           const double *x, size_t xstart, size_t xinc, double alpha,
                           double beta, double *y, size_t ystart, size_t yinc) {
  long r;
#pragma omp parallel for if (n > VO_OMP_MIN)
  for (r = 0; r < (long)n; ++r) {
    double acc = 0;
    vo_u32 k;
    for (k = rp[r]; k < rp[r + 1]; ++k) acc += v[k] * x[(size_t)ci[k] * xinc + xstart];
    size_t idx = (size_t)r * yinc + ystart;
    if (beta < 0 || beta > 0)
      y[idx] = alpha * acc + beta * y[idx];
    else
      y[idx] = alpha * acc;
  }
}

/* row_info(SPARSE_ROW_DIAGONAL) -- host_based/sparse_matrix_operations.hpp:52-98 */
#define VO_DEF_DIAG(T, S)                                                                 \
  void vo_csr_diag_##S(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const T *v, T *d) { \
    vo_u32 r, k;                                                                          \
    for (r = 0; r < n; ++r) {                                                             \
      T val = 0;                                                                          \
      for (k = rp[r]; k < rp[r + 1]; ++k)                                                 \
        if (ci[k] == r) { val = v[k]; break; }                                            \
      d[r] = val;                                                                         \
    }                                                                                     \
  }
VO_DEF_DIAG(double, d)
VO_DEF_DIAG(float, s)

/* row_info(SPARSE_ROW_NORM_INF / _1 / _2) -- host_based/sparse_matrix_operations.hpp:52-98,
 * the diagonal of row_scaling (linalg/row_scaling.hpp:166-182) */
void vo_row_norms_d(vo_u32 n, const vo_u32 *rp, const double *v, vo_u32 norm, double *d) {
  for (vo_u32 r = 0; r < n; ++r) {
    double value = 0;
    for (vo_u32 k = rp[r]; k < rp[r + 1]; ++k) {
      if (norm == 0) value = value < fabs(v[k]) ? fabs(v[k]) : value;
      else if (norm == 1) value += fabs(v[k]);
      else value += v[k] * v[k];
    }
    d[r] = norm == 2 ? sqrt(value) : value;
  }
}

/* compressed_matrix::generate_row_block_information -- compressed_matrix.hpp:1152-1188.
 * Greedy blocks of at most 1024 entries; a row longer than that forms its own
 * block; a trailing run of empty rows after a boundary gets no block. */
size_t vo_csr_row_blocks(vo_u32 n, const vo_u32 *rp, vo_u32 *blocks) {
  const size_t cap = 1024;
  size_t num = 0, count = 0;
  long i;
  blocks[0] = 0;
  for (i = 0; i < (long)n; ++i) {
    count += (size_t)(rp[i + 1] - rp[i]);
    if (count > cap) {
      size_t rows_in_batch = (size_t)i - blocks[num];
      if (rows_in_batch > 0) {
        blocks[++num] = (vo_u32)i;
        --i;
      } else {
        blocks[++num] = (vo_u32)(i + 1);
      }
      count = 0;
    }
  }
  if (count > 0) blocks[++num] = n;
  return num;
}

/* ------------------------------------------------------------------------ */
/* ELL -- ell_matrix.hpp:123-171 (copy), host SpMV sparse_matrix_operations.hpp:1502-1538 */
/* ------------------------------------------------------------------------ */
vo_u32 vo_ell_width(vo_u32 n, const vo_u32 *rp) {
  vo_u32 w = 0, r;
  for (r = 0; r < n; ++r) {
    vo_u32 l = rp[r + 1] - rp[r];
    if (l > w) w = l;
  }
  return w;
}

void vo_ell_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, vo_u32 width,
                   vo_u32 *coords, double *elems) {
  size_t total = (size_t)n * width;
  memset(coords, 0, total * sizeof(vo_u32));
  memset(elems, 0, total * sizeof(double));
  for (vo_u32 r = 0; r < n; ++r) {
    size_t item = 0;
    for (vo_u32 k = rp[r]; k < rp[r + 1]; ++k, ++item) {
      coords[item * n + r] = ci[k];
      elems[item * n + r] = v[k];
    }
  }
}

/* host ELL SpMV skips explicit zeros (val != 0) -- sparse_matrix_operations.hpp:1518-1530 */
void vo_ell_spmv_d(vo_u32 n, vo_u32 width, const vo_u32 *coords, const double *elems,
                   const double *x, double alpha, double beta, double *y) {
  long r;
#pragma omp parallel for if (n > VO_OMP_MIN)
  for (r = 0; r < (long)n; ++r) {
    double acc = 0;
    for (vo_u32 item = 0; item < width; ++item) {
      size_t off = (size_t)item * n + (size_t)r;
      double val = elems[off];
      if (val < 0 || val > 0) acc += val * x[coords[off]];
    }
    if (beta < 0 || beta > 0)
      y[r] = alpha * acc + beta * y[r];
    else
      y[r] = alpha * acc;
  }
}

/* ------------------------------------------------------------------------ */
/* SELL-C-sigma -- sliced_ell_matrix.hpp:140-214 (copy, sigma = 1).          */
/* For sigma > 1 rows are stably sorted by decreasing length inside windows  */
/* of sigma rows (Kreutzer et al. 2014, cited at sliced_ell_matrix.hpp:39);  */
/* the reference has no sigma > 1 code, so this restatement is the oracle.   */
/* ------------------------------------------------------------------------ */
typedef struct { vo_u32 len, row; } vo_lenrow;
static int vo_cmp_len_desc(const void *a, const void *b) {
  const vo_lenrow *x = (const vo_lenrow *)a, *y = (const vo_lenrow *)b;
  if (x->len != y->len) return x->len > y->len ? -1 : 1;
  return x->row < y->row ? -1 : (x->row > y->row ? 1 : 0); /* stable */
}

size_t vo_sell_layout(vo_u32 n, const vo_u32 *rp, vo_u32 C, vo_u32 sigma, vo_u32 *perm,
                      vo_u32 *columns_per_block, vo_u32 *block_start) {
  vo_u32 r;
  if (n == 0) return 0;
  if (sigma <= 1) {
    for (r = 0; r < n; ++r) perm[r] = r;
  } else {
    vo_lenrow *tmp = (vo_lenrow *)malloc(sizeof(vo_lenrow) * sigma);
    for (vo_u32 w0 = 0; w0 < n; w0 += sigma) {
      vo_u32 w1 = w0 + sigma < n ? w0 + sigma : n;
      for (r = w0; r < w1; ++r) { tmp[r - w0].len = rp[r + 1] - rp[r]; tmp[r - w0].row = r; }
      qsort(tmp, w1 - w0, sizeof(vo_lenrow), vo_cmp_len_desc);
      for (r = w0; r < w1; ++r) perm[r] = tmp[r - w0].row;
    }
    free(tmp);
  }
  vo_u32 nslices = (n - 1) / C + 1;
  size_t offset = 0;
  for (vo_u32 s = 0; s < nslices; ++s) {
    vo_u32 w = 0;
    for (vo_u32 l = 0; l < C; ++l) {
      vo_u32 pos = s * C + l;
      if (pos >= n) break;
      vo_u32 row = perm[pos];
      vo_u32 len = rp[row + 1] - rp[row];
      if (len > w) w = len;
    }
    columns_per_block[s] = w;
    block_start[s] = (vo_u32)offset;
    offset += (size_t)w * C;
  }
  return offset;
}

void vo_sell_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, vo_u32 C,
                    const vo_u32 *perm, const vo_u32 *columns_per_block,
                    const vo_u32 *block_start, vo_u32 *coords, double *elems) {
  if (n == 0) return;
  vo_u32 nslices = (n - 1) / C + 1;
  size_t total = (size_t)block_start[nslices - 1] + (size_t)columns_per_block[nslices - 1] * C;
  memset(coords, 0, total * sizeof(vo_u32));
  memset(elems, 0, total * sizeof(double));
  for (vo_u32 pos = 0; pos < n; ++pos) {
    vo_u32 s = pos / C, l = pos % C, row = perm[pos];
    size_t j = 0;
    for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k, ++j) {
      size_t idx = (size_t)block_start[s] + j * C + l;
      coords[idx] = ci[k];
      elems[idx] = v[k];
    }
  }
}

/* SELL SpMV, restated from the intent of host_based/sparse_matrix_operations.hpp:1796-1858
 * but bounded by the real number of slices ((n-1)/C+1): the host loop there reads one
 * slice past the end when n % C == 0. */
void vo_sell_spmv_d(vo_u32 n, vo_u32 C, const vo_u32 *perm, const vo_u32 *columns_per_block,
                    const vo_u32 *block_start, const vo_u32 *coords, const double *elems,
                    const double *x, double alpha, double beta, double *y) {
  if (n == 0) return;
  long nslices = (long)((n - 1) / C + 1), s;
#pragma omp parallel for if (n > VO_OMP_MIN)
  for (s = 0; s < nslices; ++s) {
    for (vo_u32 l = 0; l < C; ++l) {
      vo_u32 pos = (vo_u32)s * C + l;
      if (pos >= n) break;
      double acc = 0;
      for (vo_u32 j = 0; j < columns_per_block[s]; ++j) {
        size_t idx = (size_t)block_start[s] + (size_t)j * C + l;
        double val = elems[idx];
        if (val < 0 || val > 0) acc += val * x[coords[idx]];
      }
      vo_u32 row = perm[pos];
      if (beta < 0 || beta > 0)
        y[row] = alpha * acc + beta * y[row];
      else
        y[row] = alpha * acc;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* HYB -- hyb_matrix.hpp:135-234 (copy), host SpMV sparse_matrix_operations.hpp:1872-1927 */
/* ------------------------------------------------------------------------ */
vo_u32 vo_hyb_width(vo_u32 n, vo_u32 ncols, const vo_u32 *rp, double threshold, int is_float,
                    size_t *tail_nnz) {
  size_t *hist = (size_t *)calloc((size_t)ncols + 2, sizeof(size_t));
  vo_u32 maxl = 0, r;
  for (r = 0; r < n; ++r) {
    vo_u32 l = rp[r + 1] - rp[r];
    if (l > ncols) l = ncols; /* cannot happen without duplicates */
    hist[l] += 1;
    if (l > maxl) maxl = l;
  }
  vo_u32 w = maxl;
  size_t sum = 0;
  for (vo_u32 ind = 0; ind <= maxl; ++ind) {
    sum += hist[ind];
    int hit;
    if (is_float)
      hit = (float)sum >= (float)threshold * (float)n;
    else
      hit = (double)sum >= threshold * (double)n;
    if (hit) { w = ind; break; }
  }
  free(hist);
  if (tail_nnz) {
    size_t t = 0;
    for (r = 0; r < n; ++r) {
      vo_u32 l = rp[r + 1] - rp[r];
      if (l > w) t += l - w;
    }
    *tail_nnz = t;
  }
  return w;
}

void vo_hyb_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, vo_u32 width,
                   vo_u32 *ell_coords, double *ell_elems, vo_u32 *tail_rp, vo_u32 *tail_ci,
                   double *tail_v) {
  size_t total = (size_t)n * width, t = 0;
  if (total) {
    memset(ell_coords, 0, total * sizeof(vo_u32));
    memset(ell_elems, 0, total * sizeof(double));
  }
  for (vo_u32 r = 0; r < n; ++r) {
    tail_rp[r] = (vo_u32)t;
    vo_u32 j = 0;
    for (vo_u32 k = rp[r]; k < rp[r + 1]; ++k, ++j) {
      if (j < width) {
        ell_coords[(size_t)j * n + r] = ci[k];
        ell_elems[(size_t)j * n + r] = v[k];
      } else {
        tail_ci[t] = ci[k];
        tail_v[t] = v[k];
        ++t;
      }
    }
  }
  tail_rp[n] = (vo_u32)t;
  if (t == 0) { tail_ci[0] = 0; tail_v[0] = 0; } /* placeholder, hyb_matrix.hpp:213-217 */
}

void vo_hyb_spmv_d(vo_u32 n, vo_u32 width, const vo_u32 *ell_coords, const double *ell_elems,
                   const vo_u32 *tail_rp, const vo_u32 *tail_ci, const double *tail_v,
                   const double *x, double alpha, double beta, double *y) {
  long r;
#pragma omp parallel for if (n > VO_OMP_MIN)
  for (r = 0; r < (long)n; ++r) {
    double acc = 0;
    for (vo_u32 j = 0; j < width; ++j) {
      size_t off = (size_t)j * n + (size_t)r;
      double val = ell_elems[off];
      if (val < 0 || val > 0) acc += val * x[ell_coords[off]];
    }
    for (vo_u32 k = tail_rp[r]; k < tail_rp[r + 1]; ++k) acc += tail_v[k] * x[tail_ci[k]];
    if (beta < 0 || beta > 0)
      y[r] = alpha * acc + beta * y[r];
    else
      y[r] = alpha * acc;
  }
}

/* ------------------------------------------------------------------------ */
/* COO -- coordinate_matrix.hpp:46-101 (copy), host SpMV                     */
/* host_based/sparse_matrix_operations.hpp:1222-1245                         */
/* ------------------------------------------------------------------------ */
/* coords u32[2*stored], elems[stored], groups u32[65]; stored = nnz rounded up
 * to AlignmentV = 128 (coordinate_matrix.hpp:363), padding zero.  The group
 * loop follows coordinate_matrix.hpp:74-91 literally, including its cast of
 * (f+1)/64.0 to an integer before the multiplication by nnz. */
size_t vo_coo_fill_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                     vo_u32 *coords, double *elems, vo_u32 *groups) {
  size_t nnz = rp[n], stored = (nnz + 127) / 128 * 128;
  size_t data_index = 0, f = 0;
  if (stored) {
    memset(coords, 0, 2 * stored * sizeof(vo_u32));
    memset(elems, 0, stored * sizeof(double));
  }
  memset(groups, 0, 65 * sizeof(vo_u32));
  for (vo_u32 r = 0; r < n; ++r) {
    for (vo_u32 k = rp[r]; k < rp[r + 1]; ++k) {
      coords[2 * data_index] = r;
      coords[2 * data_index + 1] = ci[k];
      elems[data_index] = v[k];
      ++data_index;
    }
    while (data_index > (size_t)((double)(f + 1) / 64.0) * nnz) groups[++f] = (vo_u32)data_index;
  }
  groups[64] = (vo_u32)data_index;
  return stored;
}

/* y = beta*y (or 0), then y[row] += alpha*e*x[col] entry by entry (sequential) */
void vo_coo_spmv_d(vo_u32 n, size_t nnz, const vo_u32 *coords, const double *elems,
                   const double *x, double alpha, double beta, double *y) {
  for (vo_u32 i = 0; i < n; ++i) y[i] = (beta < 0 || beta > 0) ? y[i] * beta : 0.0;
  for (size_t k = 0; k < nnz; ++k) y[coords[2 * k]] += alpha * elems[k] * x[coords[2 * k + 1]];
}

/* ------------------------------------------------------------------------ */
/* vector kernels (host_based/vector_operations.hpp)                        */
/* ------------------------------------------------------------------------ */
double vo_dot_d(size_t n, const double *a, const double *b) {
  double s = 0;
  long i;
#pragma omp parallel for reduction(+ : s) if (n > VO_OMP_MIN)
  for (i = 0; i < (long)n; ++i) s += a[i] * b[i];
  return s;
}

static float vo_dot_s(size_t n, const float *a, const float *b) {
  float s = 0;
  long i;
#pragma omp parallel for reduction(+ : s) if (n > VO_OMP_MIN)
  for (i = 0; i < (long)n; ++i) s += a[i] * b[i];
  return s;
}

double vo_rel_residual_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                         const double *x, const double *b) {
  double *r = (double *)malloc(sizeof(double) * (n ? n : 1));
  vo_csr_spmv_d(n, rp, ci, v, x, 1.0, 0.0, r);
  double rr = 0, bb = 0;
  long i;
#pragma omp parallel for reduction(+ : rr, bb) if (n > VO_OMP_MIN)
  for (i = 0; i < (long)n; ++i) {
    double d = b[i] - r[i];
    rr += d * d;
    bb += b[i] * b[i];
  }
  free(r);
  return bb > 0 ? sqrt(rr / bb) : sqrt(rr);
}

/* ------------------------------------------------------------------------ */
/* preconditioners                                                          */
/* ------------------------------------------------------------------------ */
/* ILU0 substitution without level scheduling: unit-lower then upper CSR solves,
 * host_based/sparse_matrix_operations.hpp csr_inplace_solve (unit_lower_tag,
 * upper_tag) as called by ilu0_precond::apply (detail/ilu/ilu0.hpp:164-172). */
static void vo_ilu0_solve(vo_u32 n, const vo_precond *P, double *vec) {
  for (vo_u32 r = 0; r < n; ++r) {
    double s = vec[r];
    for (vo_u32 k = P->rp[r]; k < P->rp[r + 1]; ++k)
      if (P->ci[k] < r) s -= P->lu[k] * vec[P->ci[k]];
    vec[r] = s;
  }
  for (long r = (long)n - 1; r >= 0; --r) {
    double s = vec[r], diag = 0;
    for (vo_u32 k = P->rp[r]; k < P->rp[r + 1]; ++k) {
      if (P->ci[k] > (vo_u32)r)
        s -= P->lu[k] * vec[P->ci[k]];
      else if (P->ci[k] == (vo_u32)r)
        diag = P->lu[k];
    }
    vec[r] = s / diag;
  }
}

/* jacobi_precond::apply = element_div(vec, diag) -- jacobi_precond.hpp:121-126 */
/* ------------------------------------------------------------------------ */
/* block ILU0: block_ilu_precond<compressed_matrix, ilu0_tag>                */
/* (linalg/detail/ilu/block_ilu.hpp:322-573) keeps each block's LU as both   */
/* L and U, moves it into L^T / U^T / D and solves column by column          */
/* (host_based/sparse_matrix_operations.hpp:868-896, 968-1000).  Restated    */
/* by rows: x_r -= x_c l_rc for c < r ascending, then from the last row up   */
/* x_r -= x_c u_rc for c > r descending and x_r /= d_r -- the same           */
/* operations in the same order as the column sweeps.                        */
/* ------------------------------------------------------------------------ */
/* The reference never writes U^T's last row pointer (the exclusive scans of
 * block_ilu.hpp:460-475 stop at size1 - 1 and reserve() leaves the end at 0),
 * so its column sweep skips U's last column.  The quirk switch reproduces that
 * to pin this restatement against the reference's outputs; off (the default),
 * every entry of U is applied, as the engine does. */
static int vo_block_ilu_quirk = 0;
void vo_set_block_ilu_host_quirk(int on) { vo_block_ilu_quirk = on; }

void vo_block_ilu0_apply_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *lu,
                           double *vec) {
  const vo_u32 skip_col = vo_block_ilu_quirk && n ? n - 1 : 0xffffffffu;
  for (vo_u32 r = 0; r < n; ++r)
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j)
      if (ci[j] < r) vec[r] -= vec[ci[j]] * lu[j];
  for (vo_u32 r2 = 0; r2 < n; ++r2) {
    vo_u32 r = n - 1 - r2;
    double d = 0; /* D stays 0 for a row without a diagonal entry */
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j)
      if (ci[j] == r) d = lu[j];
    for (vo_u32 j = rp[r + 1]; j > rp[r]; --j)
      if (ci[j - 1] > r && ci[j - 1] != skip_col) vec[r] -= vec[ci[j - 1]] * lu[j - 1];
    vec[r] = vec[r] / d;
  }
}

/* ------------------------------------------------------------------------ */
/* Chow-Patel parallel ILU0 / ICC0: linalg/detail/ilu/chow_patel_ilu.hpp     */
/* (setup :77-150, apply :190-222 and :269-300) over the host kernels of     */
/* linalg/host_based/ilu_operations.hpp.  Sweeps read the previous sweep's  */
/* values only (the reference's backup copies), so they are deterministic.  */
/* ------------------------------------------------------------------------ */
void vo_cp_counts(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, size_t *nnz_l, size_t *nnz_u) {
  size_t l = 0, u = 0;
  for (vo_u32 r = 0; r < n; ++r)
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j) {
      if (ci[j] <= r) ++l;
      if (ci[j] >= r) ++u;
    }
  *nnz_l = l;
  *nnz_u = u;
}

/* extract_L / extract_LU (ilu_operations.hpp:52-121, 257-345): a row's lower
 * (col <= row) or upper (col >= row) entries in storage order */
static void vo_cp_extract(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                          int upper, vo_u32 *orp, vo_u32 *oci, double *ov) {
  size_t k = 0;
  orp[0] = 0;
  for (vo_u32 r = 0; r < n; ++r) {
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j)
      if (upper ? ci[j] >= r : ci[j] <= r) {
        oci[k] = ci[j];
        ov[k] = v[j];
        ++k;
      }
    orp[r + 1] = (vo_u32)k;
  }
}

/* ilu_scale / icc_scale (:123-182, :348-428): D_r = 1 / sqrt(|a_rr|) from the
 * row's first diagonal entry (0 without one), then m_ij *= D_i * D_j */
static void vo_cp_scale_vector(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                               double *D) {
  for (vo_u32 r = 0; r < n; ++r) {
    D[r] = 0;
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j)
      if (ci[j] == r) {
        D[r] = 1.0 / sqrt(fabs(v[j]));
        break;
      }
  }
}

static void vo_cp_scale(vo_u32 n, const vo_u32 *mrp, const vo_u32 *mci, double *mv,
                        const double *D) {
  for (vo_u32 r = 0; r < n; ++r) {
    double dr = D[r];
    for (vo_u32 j = mrp[r]; j < mrp[r + 1]; ++j) mv[j] *= dr * D[mci[j]];
  }
}

/* ilu_transpose (:430-500): rows of the transpose in ascending source row */
static void vo_cp_transpose(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                            vo_u32 *trp, vo_u32 *tci, double *tv) {
  vo_u32 *cur = (vo_u32 *)calloc((size_t)n + 1, sizeof(vo_u32));
  for (vo_u32 c = 0; c <= n; ++c) trp[c] = 0;
  for (vo_u32 r = 0; r < n; ++r)
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j) trp[ci[j]] += 1;
  vo_u32 off = 0;
  for (vo_u32 c = 0; c < n; ++c) {
    vo_u32 t = trp[c];
    trp[c] = off;
    off += t;
  }
  trp[n] = off;
  for (vo_u32 r = 0; r < n; ++r)
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j) {
      vo_u32 c = ci[j], k = trp[c] + cur[c]++;
      tci[k] = r;
      tv[k] = v[j];
    }
  free(cur);
}

/* ilu_chow_patel_sweep (:502-623): L from the previous L and U^T, U^T from the
 * previous L and U^T; l_ij = (a_ij - sum_k l_ik u_kj) / u_jj, u_ij = a_ij - sum */
static void vo_cp_ilu_sweep(vo_u32 n, const vo_u32 *lrp, const vo_u32 *lci, double *lv,
                            const double *aL, const vo_u32 *utrp, const vo_u32 *utci, double *utv,
                            const double *aU, double *Lb, double *Ub) {
  long row;
  memcpy(Lb, lv, sizeof(double) * lrp[n]);
  memcpy(Ub, utv, sizeof(double) * utrp[n]);
#pragma omp parallel for if (n > VO_OMP_MIN)
  for (row = 0; row < (long)n; ++row) {
    vo_u32 ls = lrp[row], le = lrp[row + 1];
    for (vo_u32 j = ls; j < le; ++j) {
      vo_u32 col = lci[j];
      if (col == (vo_u32)row) continue;
      vo_u32 us = utrp[col], ue = utrp[col + 1], iu = us;
      vo_u32 cu = iu < ue ? utci[iu] : n;
      double sum = 0;
      for (vo_u32 k = ls; k < j; ++k) {
        vo_u32 cl = lci[k];
        while (cu < cl) cu = utci[++iu];
        if (cu == cl) sum += Lb[k] * Ub[iu];
      }
      lv[j] = (aL[j] - sum) / Ub[ue - 1];
    }
    vo_u32 us = utrp[row], ue = utrp[row + 1];
    for (vo_u32 j = us; j < ue; ++j) {
      vo_u32 col = utci[j];
      vo_u32 cs = lrp[col], ce = lrp[col + 1], il = cs;
      vo_u32 cl = il < ce ? lci[il] : n;
      double sum = 0;
      for (vo_u32 k = us; k < j; ++k) {
        vo_u32 cu = utci[k];
        while (cl < cu) cl = lci[++il];
        if (cu == cl) sum += Lb[il] * Ub[k];
      }
      utv[j] = aU[j] - sum;
    }
  }
}

/* icc_chow_patel_sweep (:184-255): l_ij = (a_ij - sum_k l_ik l_jk) / l_jj,
 * l_ii = sqrt(a_ii - sum_k l_ik^2) */
static void vo_cp_icc_sweep(vo_u32 n, const vo_u32 *lrp, const vo_u32 *lci, double *lv,
                            const double *aL, double *Lb) {
  long row;
  memcpy(Lb, lv, sizeof(double) * lrp[n]);
#pragma omp parallel for if (n > VO_OMP_MIN)
  for (row = 0; row < (long)n; ++row) {
    vo_u32 s0 = lrp[row], e0 = lrp[row + 1];
    for (vo_u32 i = s0; i < e0; ++i) {
      vo_u32 col = lci[i];
      vo_u32 js = lrp[col], je = lrp[col + 1], ij = js;
      vo_u32 cj = lci[ij];
      double s = aL[i];
      for (vo_u32 ii = s0; ii < i; ++ii) {
        vo_u32 c = lci[ii];
        while (cj < c) cj = lci[++ij];
        if (cj == c) s -= Lb[ii] * Lb[ij];
      }
      lv[i] = col != (vo_u32)row ? s / Lb[je - 1] : sqrt(s);
    }
  }
}

/* ilu_form_neumann_matrix (:625-667): d = the row's first diagonal entry, which
 * is set to 0; every entry of the row is then divided by -d */
static void vo_cp_neumann(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, double *v, double *diag) {
  for (vo_u32 r = 0; r < n; ++r) {
    double d = 0;
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j)
      if (ci[j] == r) {
        d = v[j];
        v[j] = 0;
        break;
      }
    diag[r] = d;
    for (vo_u32 j = rp[r]; j < rp[r + 1]; ++j) v[j] /= -d;
  }
}

void vo_chow_patel_ilu_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                         vo_u32 sweeps, vo_u32 *l_rp, vo_u32 *l_ci, double *l_v, double *diag_l,
                         vo_u32 *u_rp, vo_u32 *u_ci, double *u_v, double *diag_u) {
  vo_cp_extract(n, rp, ci, v, 0, l_rp, l_ci, l_v);
  vo_cp_extract(n, rp, ci, v, 1, u_rp, u_ci, u_v);
  size_t nl = l_rp[n], nu = u_rp[n];
  double *D = (double *)malloc(sizeof(double) * (n ? n : 1));
  vo_cp_scale_vector(n, rp, ci, v, D);
  vo_cp_scale(n, l_rp, l_ci, l_v, D);
  vo_cp_scale(n, u_rp, u_ci, u_v, D);
  vo_u32 *ut_rp = (vo_u32 *)malloc(sizeof(vo_u32) * ((size_t)n + 1));
  vo_u32 *ut_ci = (vo_u32 *)malloc(sizeof(vo_u32) * (nu ? nu : 1));
  double *ut_v = (double *)malloc(sizeof(double) * (nu ? nu : 1));
  vo_cp_transpose(n, u_rp, u_ci, u_v, ut_rp, ut_ci, ut_v);
  double *aL = (double *)malloc(sizeof(double) * (nl ? nl : 1));
  double *aU = (double *)malloc(sizeof(double) * (nu ? nu : 1));
  double *Lb = (double *)malloc(sizeof(double) * (nl ? nl : 1));
  double *Ub = (double *)malloc(sizeof(double) * (nu ? nu : 1));
  memcpy(aL, l_v, sizeof(double) * nl);
  memcpy(aU, ut_v, sizeof(double) * nu);
  for (vo_u32 s = 0; s < sweeps; ++s)
    vo_cp_ilu_sweep(n, l_rp, l_ci, l_v, aL, ut_rp, ut_ci, ut_v, aU, Lb, Ub);
  vo_cp_transpose(n, ut_rp, ut_ci, ut_v, u_rp, u_ci, u_v);
  vo_cp_neumann(n, l_rp, l_ci, l_v, diag_l);
  vo_cp_neumann(n, u_rp, u_ci, u_v, diag_u);
  free(D); free(ut_rp); free(ut_ci); free(ut_v); free(aL); free(aU); free(Lb); free(Ub);
}

void vo_chow_patel_icc_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                         vo_u32 sweeps, vo_u32 *l_rp, vo_u32 *l_ci, double *l_v,
                         vo_u32 *lt_rp, vo_u32 *lt_ci, double *lt_v, double *diag_l) {
  vo_cp_extract(n, rp, ci, v, 0, l_rp, l_ci, l_v);
  size_t nl = l_rp[n];
  double *D = (double *)malloc(sizeof(double) * (n ? n : 1));
  vo_cp_scale_vector(n, rp, ci, v, D);
  vo_cp_scale(n, l_rp, l_ci, l_v, D);
  double *aL = (double *)malloc(sizeof(double) * (nl ? nl : 1));
  double *Lb = (double *)malloc(sizeof(double) * (nl ? nl : 1));
  memcpy(aL, l_v, sizeof(double) * nl);
  for (vo_u32 s = 0; s < sweeps; ++s) vo_cp_icc_sweep(n, l_rp, l_ci, l_v, aL, Lb);
  vo_cp_transpose(n, l_rp, l_ci, l_v, lt_rp, lt_ci, lt_v);
  vo_cp_neumann(n, l_rp, l_ci, l_v, diag_l);
  vo_cp_neumann(n, lt_rp, lt_ci, lt_v, diag_l);
  free(D); free(aL); free(Lb);
}

/* apply (chow_patel_ilu.hpp:269-300): y = L^-1 vec and then U^-1 y, each by
 * jacobi_iters steps x <- (I - D^-1 M) x + D^-1 rhs from x = D^-1 rhs */
static void vo_cp_apply(vo_u32 n, const vo_precond *P, double *vec) {
  size_t bytes = sizeof(double) * (n ? n : 1);
  double *b = (double *)malloc(bytes), *x = (double *)malloc(bytes);
  for (int tri = 0; tri < 2; ++tri) {
    const double *d = tri ? P->udiag : P->diag;
    const vo_u32 *mrp = tri ? P->u_rp : P->l_rp, *mci = tri ? P->u_ci : P->l_ci;
    const double *mv = tri ? P->u_v : P->l_v;
    const double *src = tri ? x : vec;
    for (vo_u32 i = 0; i < n; ++i) b[i] = src[i] / d[i];
    memcpy(x, b, sizeof(double) * n);
    for (vo_u32 it = 0; it < P->jacobi_iters; ++it) {
      vo_csr_spmv_d(n, mrp, mci, mv, x, 1.0, 0.0, vec);
      for (vo_u32 i = 0; i < n; ++i) x[i] = vec[i] + b[i];
    }
  }
  memcpy(vec, x, sizeof(double) * n);
  free(b);
  free(x);
}

void vo_precond_apply_d(vo_u32 n, const vo_precond *P, double *vec) {
  if (!P || P->kind == VO_PRECOND_NONE) return;
  if (P->kind == VO_PRECOND_JACOBI) {
    long i;
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) vec[i] = vec[i] / P->diag[i];
  } else if (P->kind == VO_PRECOND_ILU0) {
    vo_ilu0_solve(n, P, vec);
  } else if (P->kind == VO_PRECOND_CHOW_PATEL) {
    vo_cp_apply(n, P, vec);
  } else if (P->kind == VO_PRECOND_BLOCK_ILU0) {
    vo_block_ilu0_apply_d(n, P->rp, P->ci, P->lu, vec);
  }
}

/* ------------------------------------------------------------------------ */
/* CG                                                                       */
/* ------------------------------------------------------------------------ */
/* pipelined CG, cg.hpp:128-187, with the fused host kernels of
 * host_based/iterative_operations.hpp:52-105 (prod + <Ap,Ap>, <p,Ap>) and
 * :378-416 (x += a p; r -= a Ap; p = r + b p; <r,r>). */
static void vo_cg_pipelined(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                            const double *b, double *x, vo_tag *tag) {
  size_t bytes = sizeof(double) * (n ? n : 1);
  double *r = (double *)malloc(bytes), *p = (double *)malloc(bytes), *Ap = (double *)malloc(bytes);
  memset(x, 0, sizeof(double) * n);
  memcpy(r, b, sizeof(double) * n);
  memcpy(p, b, sizeof(double) * n);
  vo_csr_spmv_d(n, rp, ci, v, p, 1.0, 0.0, Ap);
  double nrm = sqrt(vo_dot_d(n, r, r));
  double norm_rhs_squared = nrm * nrm;
  tag->iters = 0;
  tag->error = 0;
  if (norm_rhs_squared <= tag->abs_tol * tag->abs_tol) goto done;
  {
    double rr = norm_rhs_squared;
    double alpha = rr / vo_dot_d(n, p, Ap);
    double nap = sqrt(vo_dot_d(n, Ap, Ap));
    double beta = (alpha * alpha * nap * nap - rr) / rr;
    double ApAp = 0, pAp = 0;
    for (vo_u32 it = 0; it < tag->max_iters; ++it) {
      tag->iters = it + 1;
      double s_rr = 0, s_ApAp = 0, s_pAp = 0;
      long i;
#pragma omp parallel for reduction(+ : s_rr) if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) {
        double vp = p[i], vr = r[i];
        x[i] += alpha * vp;
        vr -= alpha * Ap[i];
        vp = vr + beta * vp;
        s_rr += vr * vr;
        p[i] = vp;
        r[i] = vr;
      }
#pragma omp parallel for reduction(+ : s_ApAp, s_pAp) if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) {
        double acc = 0;
        for (vo_u32 k = rp[i]; k < rp[i + 1]; ++k) acc += v[k] * p[ci[k]];
        Ap[i] = acc;
        s_ApAp += acc * acc;
        s_pAp += p[i] * acc;
      }
      rr = s_rr;
      ApAp = s_ApAp;
      pAp = s_pAp;
      if (fabs(rr / norm_rhs_squared) < tag->tol * tag->tol ||
          fabs(rr) < tag->abs_tol * tag->abs_tol)
        break;
      alpha = rr / pAp;
      beta = (alpha * alpha * ApAp - rr) / rr;
    }
    tag->error = sqrt(fabs(rr) / norm_rhs_squared);
  }
done:
  free(r);
  free(p);
  free(Ap);
}

/* preconditioned CG, cg.hpp:257-322 (Saad Alg. 9.1) */
static void vo_cg_precond(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                          const double *b, double *x, vo_tag *tag, const vo_precond *P) {
  size_t bytes = sizeof(double) * (n ? n : 1);
  double *r = (double *)malloc(bytes), *z = (double *)malloc(bytes), *p = (double *)malloc(bytes),
         *tmp = (double *)malloc(bytes);
  memset(x, 0, sizeof(double) * n);
  memcpy(r, b, sizeof(double) * n);
  memcpy(z, r, sizeof(double) * n);
  vo_precond_apply_d(n, P, z);
  memcpy(p, z, sizeof(double) * n);
  double ip_rr = vo_dot_d(n, r, z);
  double norm_rhs_squared = ip_rr, new_ip_rr = 0;
  tag->iters = 0;
  tag->error = 0;
  if (fabs(norm_rhs_squared) <= tag->abs_tol * tag->abs_tol) goto done;
  for (vo_u32 it = 0; it < tag->max_iters; ++it) {
    tag->iters = it + 1;
    vo_csr_spmv_d(n, rp, ci, v, p, 1.0, 0.0, tmp);
    double alpha = ip_rr / vo_dot_d(n, tmp, p);
    long i;
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) x[i] += alpha * p[i];
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) r[i] -= alpha * tmp[i];
    memcpy(z, r, sizeof(double) * n);
    vo_precond_apply_d(n, P, z);
    new_ip_rr = vo_dot_d(n, r, z);
    double ratio = new_ip_rr / norm_rhs_squared;
    if (fabs(ratio) < tag->tol * tag->tol || fabs(new_ip_rr) < tag->abs_tol * tag->abs_tol) break;
    double beta = new_ip_rr / ip_rr;
    ip_rr = new_ip_rr;
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) p[i] = z[i] + beta * p[i];
  }
  tag->error = sqrt(fabs(new_ip_rr / norm_rhs_squared));
done:
  free(r);
  free(z);
  free(p);
  free(tmp);
}

void vo_cg_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
             double *x, vo_tag *tag, const vo_precond *P) {
  if (!P || P->kind == VO_PRECOND_NONE)
    vo_cg_pipelined(n, rp, ci, v, b, x, tag);
  else
    vo_cg_precond(n, rp, ci, v, b, x, tag, P);
}

/* ------------------------------------------------------------------------ */
/* BiCGStab                                                                 */
/* ------------------------------------------------------------------------ */
/* pipelined BiCGStab, bicgstab.hpp:96-215 with host_based/iterative_operations.hpp:519-627.
 * As in the reference, the loop leaves on convergence before the final update of x. */
static void vo_bicgstab_pipelined(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                                  const double *b, double *x, vo_tag *tag) {
  size_t bytes = sizeof(double) * (n ? n : 1);
  double *r = (double *)malloc(bytes), *p = (double *)malloc(bytes), *r0 = (double *)malloc(bytes),
         *Ap = (double *)malloc(bytes), *s = (double *)malloc(bytes), *As = (double *)malloc(bytes);
  memset(x, 0, sizeof(double) * n);
  memcpy(r, b, sizeof(double) * n);
  memcpy(p, b, sizeof(double) * n);
  memcpy(r0, b, sizeof(double) * n);
  double norm_rhs = sqrt(vo_dot_d(n, r, r));
  double residual_norm = norm_rhs;
  double r_dot_r0 = norm_rhs * norm_rhs;
  tag->iters = 0;
  tag->error = 0;
  if (norm_rhs <= tag->abs_tol) goto done;
  for (vo_u32 it = 0; it < tag->max_iters; ++it) {
    tag->iters = it + 1;
    double Ap_dot_r0 = 0, s_dot_s = 0, As_dot_As = 0, As_dot_s = 0, As_dot_r0 = 0;
    long i;
    /* Ap = A p, <Ap, r0*> */
#pragma omp parallel for reduction(+ : Ap_dot_r0) if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) {
      double acc = 0;
      for (vo_u32 k = rp[i]; k < rp[i + 1]; ++k) acc += v[k] * p[ci[k]];
      Ap[i] = acc;
      Ap_dot_r0 += acc * r0[i];
    }
    /* update_s: alpha from chunks 0 and 3, s = r - alpha Ap, <s,s> */
    double alpha = r_dot_r0 / Ap_dot_r0;
#pragma omp parallel for reduction(+ : s_dot_s) if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) {
      double vs = r[i] - alpha * Ap[i];
      s_dot_s += vs * vs;
      s[i] = vs;
    }
    /* As = A s, <As,As>, <s,As>, <As,r0*> */
#pragma omp parallel for reduction(+ : As_dot_As, As_dot_s, As_dot_r0) if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) {
      double acc = 0;
      for (vo_u32 k = rp[i]; k < rp[i + 1]; ++k) acc += v[k] * s[ci[k]];
      As[i] = acc;
      As_dot_As += acc * acc;
      As_dot_s += s[i] * acc;
      As_dot_r0 += acc * r0[i];
    }
    alpha = r_dot_r0 / Ap_dot_r0;
    double beta = -As_dot_r0 / Ap_dot_r0;
    double omega = As_dot_s / As_dot_As;
    residual_norm = sqrt(s_dot_s - 2.0 * omega * As_dot_s + omega * omega * As_dot_As);
    if (fabs(residual_norm / norm_rhs) < tag->tol || residual_norm < tag->abs_tol) break;
    double rr0 = 0;
#pragma omp parallel for reduction(+ : rr0) if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) {
      double vp = p[i];
      x[i] += alpha * vp + omega * s[i];
      double vr = s[i] - omega * As[i];
      vp = vr + beta * (vp - omega * Ap[i]);
      rr0 += vr * r0[i];
      r[i] = vr;
      p[i] = vp;
    }
    r_dot_r0 = rr0;
  }
  tag->error = residual_norm / norm_rhs;
done:
  free(r); free(p); free(r0); free(Ap); free(s); free(As);
}

/* preconditioned BiCGStab, bicgstab.hpp:398-489 */
static void vo_bicgstab_precond(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                                const double *b, double *x, vo_tag *tag, const vo_precond *P) {
  size_t bytes = sizeof(double) * (n ? n : 1);
  double *r = (double *)malloc(bytes), *r0 = (double *)malloc(bytes), *t0 = (double *)malloc(bytes),
         *t1 = (double *)malloc(bytes), *s = (double *)malloc(bytes), *p = (double *)malloc(bytes);
  memset(x, 0, sizeof(double) * n);
  memcpy(r, b, sizeof(double) * n);
  double norm_rhs = sqrt(vo_dot_d(n, r, r));
  double ip_rr0 = norm_rhs, residual_norm = norm_rhs;
  tag->iters = 0;
  tag->error = 0;
  if (norm_rhs <= tag->abs_tol) goto done;
  {
    int restart = 1;
    vo_u32 last_restart = 0;
    for (vo_u32 it = 0; it < tag->max_iters; ++it) {
      long i;
      if (restart) {
        vo_csr_spmv_d(n, rp, ci, v, x, 1.0, 0.0, r);
#pragma omp parallel for if (n > VO_OMP_MIN)
        for (i = 0; i < (long)n; ++i) r[i] = b[i] - r[i];
        vo_precond_apply_d(n, P, r);
        memcpy(p, r, sizeof(double) * n);
        memcpy(r0, r, sizeof(double) * n);
        double nr = sqrt(vo_dot_d(n, r, r));
        ip_rr0 = nr * nr;
        restart = 0;
        last_restart = it;
      }
      tag->iters = it + 1;
      vo_csr_spmv_d(n, rp, ci, v, p, 1.0, 0.0, t0);
      vo_precond_apply_d(n, P, t0);
      double alpha = ip_rr0 / vo_dot_d(n, t0, r0);
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) s[i] = r[i] - alpha * t0[i];
      vo_csr_spmv_d(n, rp, ci, v, s, 1.0, 0.0, t1);
      vo_precond_apply_d(n, P, t1);
      double nt1 = sqrt(vo_dot_d(n, t1, t1));
      double omega = vo_dot_d(n, t1, s) / (nt1 * nt1);
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) x[i] += alpha * p[i] + omega * s[i];
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) r[i] = s[i] - omega * t1[i];
      residual_norm = sqrt(vo_dot_d(n, r, r));
      if (residual_norm / norm_rhs < tag->tol || residual_norm < tag->abs_tol) break;
      double new_ip = vo_dot_d(n, r, r0);
      double beta = new_ip / ip_rr0 * alpha / omega;
      ip_rr0 = new_ip;
      if ((ip_rr0 >= 0 && ip_rr0 <= 0) || (omega >= 0 && omega <= 0) ||
          it - last_restart > tag->max_iters_before_restart)
        restart = 1;
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) p[i] = r[i] + beta * (p[i] - omega * t0[i]);
    }
  }
  tag->error = residual_norm / norm_rhs;
done:
  free(r); free(r0); free(t0); free(t1); free(s); free(p);
}

void vo_bicgstab_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
                   double *x, vo_tag *tag, const vo_precond *P) {
  if (!P || P->kind == VO_PRECOND_NONE)
    vo_bicgstab_pipelined(n, rp, ci, v, b, x, tag);
  else
    vo_bicgstab_precond(n, rp, ci, v, b, x, tag, P);
}

/* ------------------------------------------------------------------------ */
/* GMRES -- pipelined "simpler GMRES" with classical Gram-Schmidt,          */
/* gmres.hpp:181-367 and host_based/iterative_operations.hpp:734-935.       */
/* The host stage-1 kernel there drops the last vector entry from <v_i,v_k> */
/* (its per-thread range ends at work*(id+1) with work = (size-1)/threads); */
/* this restatement sums every entry, as the CUDA backend does.             */
/* ------------------------------------------------------------------------ */
/* When set, stage 1 reproduces the host kernel's partition exactly (each of T
 * threads sums [t*w, min((t+1)*w, n)) with w = (n-1)/T, so the tail past T*w
 * is dropped); used only to pin this restatement against the reference. */
static int vo_gmres_host_quirk = 0;
void vo_set_gmres_host_quirk(int on) { vo_gmres_host_quirk = on; }

static double vo_gs_dot(vo_u32 n, const double *a, const double *b) {
  if (!vo_gmres_host_quirk) return vo_dot_d(n, a, b);
  long T = vo_max_threads(), w = (long)(n - 1) / T;
  double s = 0;
  for (long t = 0; t < T; ++t) {
    double part = 0;
    long e = (t + 1) * w < (long)n ? (t + 1) * w : (long)n;
    for (long i = t * w; i < e; ++i) part += a[i] * b[i];
    s += part;
  }
  return s;
}

static vo_u32 vo_gmres_max_restarts(const vo_tag *t) {
  vo_u32 ret = t->max_iters / t->krylov_dim;
  if (ret > 0 && ret * t->krylov_dim == t->max_iters) return ret - 1;
  return ret;
}

static void vo_gmres_pipelined(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                               const double *b, double *x, vo_tag *tag) {
  vo_u32 K = tag->krylov_dim;
  size_t bytes = sizeof(double) * (n ? n : 1);
  double *r = (double *)malloc(bytes);
  double *V = (double *)malloc(bytes * K);
  double *R = (double *)calloc((size_t)K * K, sizeof(double));
  double *xi = (double *)calloc(K, sizeof(double)), *eta = (double *)calloc(K, sizeof(double));
  double *h = (double *)calloc(K, sizeof(double));
  memset(x, 0, sizeof(double) * n);
  memcpy(r, b, sizeof(double) * n);
  double norm_rhs = sqrt(vo_dot_d(n, r, r));
  double rho_0 = norm_rhs, rho = 1;
  tag->iters = 0;
  tag->error = 0;
  for (vo_u32 rc = 0; rc <= vo_gmres_max_restarts(tag); ++rc) {
    long i;
    if (rc > 0) {
      vo_csr_spmv_d(n, rp, ci, v, x, 1.0, 0.0, r);
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) r[i] = b[i] - r[i];
      rho_0 = sqrt(vo_dot_d(n, r, r));
    }
    if (rho_0 <= tag->abs_tol) break;
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) r[i] /= rho_0;
    rho = 1;
    if (rho_0 / norm_rhs < tag->tol || rho_0 < tag->abs_tol) break;

    vo_u32 k;
    for (k = 0; k < K; ++k) {
      double *vk = V + (size_t)k * n;
      const double *src = (k == 0) ? r : V + (size_t)(k - 1) * n;
      double nrm2 = 0;
#pragma omp parallel for reduction(+ : nrm2) if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) {
        double acc = 0;
        for (vo_u32 q = rp[i]; q < rp[i + 1]; ++q) acc += v[q] * src[ci[q]];
        vk[i] = acc;
        nrm2 += acc * acc;
      }
      if (k > 0) {
        /* stage 1: <v_j, v_k>, j < k */
        for (vo_u32 j = 0; j < k; ++j) h[j] = vo_gs_dot(n, V + (size_t)j * n, vk);
        /* stage 2: v_k -= sum h_j v_j; ||v_k||^2; R(j,k) = h_j */
        nrm2 = 0;
#pragma omp parallel for reduction(+ : nrm2) if (n > VO_OMP_MIN)
        for (i = 0; i < (long)n; ++i) {
          double val = vk[i];
          for (vo_u32 j = 0; j < k; ++j) val -= h[j] * V[(size_t)j * n + i];
          nrm2 += val * val;
          vk[i] = val;
        }
        for (vo_u32 j = 0; j < k; ++j) R[j + (size_t)k * K] = h[j];
      }
      /* normalize_vk: R(k,k) = ||v_k||, v_k /= ||v_k||, <r, v_k> */
      double nv = sqrt(nrm2);
      R[k + (size_t)k * K] = nv;
      double rv = 0;
#pragma omp parallel for reduction(+ : rv) if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) {
        double val = vk[i] / nv;
        rv += r[i] * val;
        vk[i] = val;
      }
      xi[k] = rv;
    }
    vo_u32 full_k = k;
    for (vo_u32 q = 0; q < k; ++q) {
      if (fabs(R[q + (size_t)q * k]) < tag->tol * R[0]) { k = q; break; }
    }
    for (vo_u32 q = 0; q < k; ++q) {
      tag->iters += 1;
      if (xi[q] >= rho || xi[q] <= -rho) { k = q; break; }
      rho *= sin(acos(xi[q] / rho));
    }
    for (vo_u32 q = 0; q < K; ++q) eta[q] = xi[q];
    for (int q2 = (int)k - 1; q2 > -1; --q2) {
      vo_u32 q = (vo_u32)q2;
      for (vo_u32 j = q + 1; j < k; ++j) eta[q] -= R[q + (size_t)j * full_k] * eta[j];
      eta[q] /= R[q + (size_t)q * full_k];
    }
    for (vo_u32 q = 0; q < k; ++q) eta[q] *= rho_0;
    /* x += c0 r + sum_{j>=1} c_j v_{j-1} */
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) {
      double val = x[i];
      if (k > 0) val += eta[0] * r[i];
      for (vo_u32 j = 1; j < k; ++j) val += eta[j] * V[(size_t)(j - 1) * n + i];
      x[i] = val;
    }
    tag->error = fabs(rho * rho_0 / norm_rhs);
  }
  free(r); free(V); free(R); free(xi); free(eta); free(h);
}

/* ------------------------------------------------------------------------ */
/* GMRES with a preconditioner -- the Householder "simpler GMRES" of        */
/* gmres.hpp:449-631 (detail::solve_impl for any preconditioner), with the  */
/* reflector set-up of gmres.hpp:131-157 and the reflection of :161-166.    */
/* Every reflection is an inner product followed by an axpy, one after the  */
/* other, as the reference applies them.                                    */
/* ------------------------------------------------------------------------ */
static void vo_hh_reflect(vo_u32 n, double *xv, const double *h, double beta) {
  double s = beta * vo_dot_d(n, h, xv);
  long i;
#pragma omp parallel for if (n > VO_OMP_MIN)
  for (i = 0; i < (long)n; ++i) xv[i] -= s * h[i];
}

/* gmres_setup_householder_vector: h = (0..0, 1, v[j+1..]/h0), beta, mu */
static void vo_hh_setup(vo_u32 n, const double *vin, double *h, double *beta, double *mu,
                        vo_u32 j) {
  double input_j = vin[j];
  memset(h, 0, sizeof(double) * n);
  for (vo_u32 i = j + 1; i < n; ++i) h[i] = vin[i];
  double sigma = sqrt(vo_dot_d(n, h, h));
  sigma *= sigma;
  if (sigma <= 0) {
    *beta = 0;
    *mu = input_j;
  } else {
    *mu = sqrt(sigma + input_j * input_j);
    double h0 = (input_j <= 0) ? (input_j - *mu) : (-sigma / (input_j + *mu));
    *beta = 2.0 * h0 * h0 / (sigma + h0 * h0);
    long i;
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) h[i] /= h0;
    h[j] = 1.0;
  }
}

/* When set, a clamp of res[k] to +-rho (gmres.hpp:575-578) ends the cycle
 * without the convergence verdict that rho = 0 gives in the reference; the
 * next restart's residual, computed from x, decides (the engine's rule). */
static int vo_gmres_clamp_restart = 0;
void vo_set_gmres_clamp_restart(int on) { vo_gmres_clamp_restart = on; }

static void vo_gmres_householder(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                                 const double *b, double *x, vo_tag *tag, const vo_precond *P) {
  vo_u32 K = tag->krylov_dim < n ? tag->krylov_dim : n;
  size_t nn = n ? n : 1;
  double *res = (double *)malloc(sizeof(double) * nn);
  double *vk = (double *)malloc(sizeof(double) * nn);
  double *tmp = (double *)malloc(sizeof(double) * nn);
  double *H = (double *)calloc(nn * (K ? K : 1), sizeof(double));
  double *R = (double *)calloc((size_t)(K ? K : 1) * (K ? K : 1), sizeof(double));
  double *proj = (double *)calloc(K ? K : 1, sizeof(double));
  double *betas = (double *)calloc(K ? K : 1, sizeof(double));
  long i;
  memset(x, 0, sizeof(double) * n);
  double norm_rhs = sqrt(vo_dot_d(n, b, b));
  tag->error = 0;
  if (norm_rhs <= tag->abs_tol) goto done;
  tag->iters = 0;
  for (vo_u32 it = 0; it <= vo_gmres_max_restarts(tag); ++it) {
    vo_csr_spmv_d(n, rp, ci, v, x, 1.0, 0.0, res);
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) res[i] = b[i] - res[i];
    vo_precond_apply_d(n, P, res);
    double rho_0 = sqrt(vo_dot_d(n, res, res));
    if (rho_0 / norm_rhs < tag->tol || rho_0 < tag->abs_tol) {
      tag->error = rho_0 / norm_rhs;
      goto done;
    }
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) res[i] /= rho_0;
    double rho = 1.0;
    int lost = 0;
    vo_u32 k;
    for (k = 0; k < K; ++k) {
      tag->iters += 1;
      double *Rk = R + (size_t)k * K, *Hk = H + (size_t)k * nn;
      memset(Rk, 0, sizeof(double) * K);
      memset(Hk, 0, sizeof(double) * nn);
      if (k == 0) {
        vo_csr_spmv_d(n, rp, ci, v, res, 1.0, 0.0, vk);
        vo_precond_apply_d(n, P, vk);
      } else {
        memset(vk, 0, sizeof(double) * n);
        vk[k - 1] = 1.0;
        for (int q = (int)k - 1; q > -1; --q) vo_hh_reflect(n, vk, H + (size_t)q * nn, betas[q]);
        vo_csr_spmv_d(n, rp, ci, v, vk, 1.0, 0.0, tmp);
        vo_precond_apply_d(n, P, tmp);
        memcpy(vk, tmp, sizeof(double) * n);
        for (vo_u32 q = 0; q < k; ++q) vo_hh_reflect(n, vk, H + (size_t)q * nn, betas[q]);
      }
      double rho_kk = 0;
      vo_hh_setup(n, vk, Hk, &betas[k], &rho_kk, k);
      for (vo_u32 q = 0; q < k; ++q) Rk[q] = vk[q];
      Rk[k] = rho_kk;
      vo_hh_reflect(n, res, Hk, betas[k]);
      int clamped = res[k] >= rho || res[k] <= -rho;
      if (res[k] > rho) res[k] = rho;
      if (res[k] < -rho) res[k] = -rho;
      proj[k] = res[k];
      rho *= sin(acos(proj[k] / rho));
      if (clamped && vo_gmres_clamp_restart) {
        lost = 1;
        ++k;
        break;
      }
      if (fabs(rho * rho_0 / norm_rhs) < tag->tol) {
        tag->error = fabs(rho * rho_0 / norm_rhs);
        ++k;
        break;
      }
    }
    /* triangular solve with R stored by columns (R[j][i] = row i of column j) */
    for (int i2 = (int)k - 1; i2 > -1; --i2) {
      vo_u32 q = (vo_u32)i2;
      for (vo_u32 j = q + 1; j < k; ++j) proj[q] -= R[(size_t)j * K + q] * proj[j];
      proj[q] /= R[(size_t)q * K + q];
    }
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) res[i] *= proj[0];
    if (k > 0)
      for (vo_u32 q = 0; q + 1 < k; ++q) res[q] += proj[q + 1];
    for (int q = (int)k - 1; q >= 0; --q) vo_hh_reflect(n, res, H + (size_t)q * nn, betas[q]);
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) x[i] += res[i] * rho_0;
    tag->error = fabs(rho * rho_0 / norm_rhs);
    if (tag->error < tag->tol && !lost) goto done;
  }
done:
  free(res); free(vk); free(tmp); free(H); free(R); free(proj); free(betas);
}

/* linalg::solve(A, b, gmres_tag[, precond]): the pipelined variant without a
 * preconditioner (gmres.hpp:369-433 dispatch), the Householder one with. */
void vo_gmres_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
                double *x, vo_tag *tag, const vo_precond *P) {
  if (!P || P->kind == VO_PRECOND_NONE)
    vo_gmres_pipelined(n, rp, ci, v, b, x, tag);
  else
    vo_gmres_householder(n, rp, ci, v, b, x, tag, P);
}

/* ------------------------------------------------------------------------ */
/* CSR triangular solves inplace_solve(A, vec, tag) and                      */
/* inplace_solve(trans(A), vec, tag): host_based/sparse_matrix_operations.hpp */
/* :537-641 (csr_inplace_solve) and :734-871 (csr_trans_inplace_solve).      */
/* tag: 0 lower, 1 upper, 2 unit_lower, 3 unit_upper.  Entries outside the   */
/* tag's strict triangle are ignored; the lower/upper forms divide by the     */
/* row's diagonal entry (the last one in the row; the transposed forms the    */
/* first one in the column's storage), 0 when absent, as the reference.      */
/* ------------------------------------------------------------------------ */
void vo_csr_inplace_solve_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                            double *vec, int tag, int trans) {
  if (!trans) {
    if (tag == 2) {  /* unit_lower: rows 1..n-1 */
      for (vo_u32 row = 1; row < n; ++row) {
        double e = vec[row];
        for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k)
          if (ci[k] < row) e -= vec[ci[k]] * v[k];
        vec[row] = e;
      }
    } else if (tag == 0) {  /* lower */
      for (vo_u32 row = 0; row < n; ++row) {
        double e = vec[row], d = 0;
        for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k) {
          if (ci[k] < row) e -= vec[ci[k]] * v[k];
          else if (ci[k] == row) d = v[k];
        }
        vec[row] = e / d;
      }
    } else if (tag == 3) {  /* unit_upper: rows n-2..0 */
      for (vo_u32 r2 = 1; r2 < n; ++r2) {
        vo_u32 row = n - r2 - 1;
        double e = vec[row];
        for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k)
          if (ci[k] > row) e -= vec[ci[k]] * v[k];
        vec[row] = e;
      }
    } else {  /* upper */
      for (vo_u32 r2 = 0; r2 < n; ++r2) {
        vo_u32 row = n - r2 - 1;
        double e = vec[row], d = 0;
        for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k) {
          if (ci[k] > row) e -= vec[ci[k]] * v[k];
          else if (ci[k] == row) d = v[k];
        }
        vec[row] = e / d;
      }
    }
    return;
  }
  /* transposed: column-oriented updates on the rows of A */
  if (tag == 2 || tag == 0) {
    for (vo_u32 col = 0; col < n; ++col) {
      double e;
      if (tag == 0) {
        double d = 0;
        for (vo_u32 k = rp[col]; k < rp[col + 1]; ++k)
          if (ci[k] == col) { d = v[k]; break; }
        e = vec[col] / d;
        vec[col] = e;
      } else {
        e = vec[col];
      }
      for (vo_u32 k = rp[col]; k < rp[col + 1]; ++k)
        if (ci[k] > col) vec[ci[k]] -= e * v[k];
    }
  } else {
    for (vo_u32 c2 = 0; c2 < n; ++c2) {
      vo_u32 col = n - c2 - 1;
      double e;
      if (tag == 1) {
        double d = 0;
        for (vo_u32 k = rp[col]; k < rp[col + 1]; ++k)
          if (ci[k] == col) { d = v[k]; break; }
        e = vec[col] / d;
        vec[col] = e;
      } else {
        e = vec[col];
      }
      for (vo_u32 k = rp[col]; k < rp[col + 1]; ++k)
        if (ci[k] < col) vec[ci[k]] -= e * v[k];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* mixed-precision CG -- mixed_precision_cg.hpp:99-186                      */
/* ------------------------------------------------------------------------ */
void vo_mixed_cg_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v, const double *b,
                   double *x, vo_tag *tag, float inner_tol) {
  size_t nn = n ? n : 1;
  double *res = (double *)malloc(sizeof(double) * nn);
  float *rl = (float *)malloc(sizeof(float) * nn), *xl = (float *)calloc(nn, sizeof(float)),
        *pl = (float *)malloc(sizeof(float) * nn), *tl = (float *)malloc(sizeof(float) * nn);
  size_t nnz = rp[n];
  float *vl = (float *)malloc(sizeof(float) * (nnz ? nnz : 1));
  for (size_t k = 0; k < nnz; ++k) vl[k] = (float)v[k];
  memset(x, 0, sizeof(double) * n);
  double ip_rr = vo_dot_d(n, b, b), new_ip_rr = 0, norm_rhs_squared = ip_rr;
  tag->iters = 0;
  tag->error = 0;
  if (norm_rhs_squared <= 0) goto done;
  {
    float inner_ip_rr = (float)ip_rr, initial = (float)ip_rr;
    long i;
    for (i = 0; i < (long)n; ++i) { pl[i] = (float)b[i]; rl[i] = pl[i]; }
    for (vo_u32 it = 0; it < tag->max_iters; ++it) {
      tag->iters = it + 1;
      vo_csr_spmv_s(n, rp, ci, vl, pl, 1.0f, 0.0f, tl);
      float alpha = inner_ip_rr / vo_dot_s(n, tl, pl);
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) xl[i] += alpha * pl[i];
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) rl[i] -= alpha * tl[i];
      float new_inner = vo_dot_s(n, rl, rl);
      float beta = new_inner / inner_ip_rr;
      inner_ip_rr = new_inner;
#pragma omp parallel for if (n > VO_OMP_MIN)
      for (i = 0; i < (long)n; ++i) pl[i] = rl[i] + beta * pl[i];
      if (new_inner < inner_tol * initial || it == tag->max_iters - 1) {
#pragma omp parallel for if (n > VO_OMP_MIN)
        for (i = 0; i < (long)n; ++i) x[i] += (double)xl[i];
        vo_csr_spmv_d(n, rp, ci, v, x, 1.0, 0.0, res);
#pragma omp parallel for if (n > VO_OMP_MIN)
        for (i = 0; i < (long)n; ++i) res[i] = b[i] - res[i];
        new_ip_rr = vo_dot_d(n, res, res);
        if (new_ip_rr / norm_rhs_squared < tag->tol * tag->tol) break;
        for (i = 0; i < (long)n; ++i) { pl[i] = (float)res[i]; xl[i] = 0; rl[i] = pl[i]; }
        initial = (float)new_ip_rr;
        inner_ip_rr = (float)new_ip_rr;
      }
    }
    tag->error = sqrt(new_ip_rr / norm_rhs_squared);
  }
done:
  free(res); free(rl); free(xl); free(pl); free(tl); free(vl);
}

/* ------------------------------------------------------------------------ */
/* FP64 iterative refinement with FP32 Jacobi-PCG inner solves.  This form  */
/* has no counterpart in the reference; it restates the engine's algorithm: */
/*   r = b - A x (FP64); stop when ||r||/||b|| < tol;                       */
/*   inner: PCG (cg.hpp:257-322 in FP32, Jacobi) on A d = r/||r|| until      */
/*   <r,z>/<r0,z0> < max(inner_tol, 0.5 tol ||b||/||r||)^2; x += ||r|| d.     */
/* ------------------------------------------------------------------------ */
void vo_ir_jacobi_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *v,
                    const double *b, double *x, double tol, vo_u32 max_outer, double inner_tol,
                    vo_u32 max_inner, vo_u32 *outer_out, vo_u32 *inner_total_out,
                    double *relres_out) {
  size_t nn = n ? n : 1, nnz = rp[n];
  double *r = (double *)malloc(sizeof(double) * nn);
  float *vl = (float *)malloc(sizeof(float) * (nnz ? nnz : 1));
  float *dl = (float *)malloc(sizeof(float) * nn), *rl = (float *)malloc(sizeof(float) * nn),
        *zl = (float *)malloc(sizeof(float) * nn), *pl = (float *)malloc(sizeof(float) * nn),
        *tl = (float *)malloc(sizeof(float) * nn), *xl = (float *)malloc(sizeof(float) * nn);
  for (size_t k = 0; k < nnz; ++k) vl[k] = (float)v[k];
  vo_csr_diag_s(n, rp, ci, vl, dl);
  memset(x, 0, sizeof(double) * n);
  memcpy(r, b, sizeof(double) * n);
  double nb = sqrt(vo_dot_d(n, b, b)), nr = nb;
  vo_u32 outer = 0, inner_total = 0;
  long i;
  while (nb > 0 && nr / nb >= tol && outer < max_outer) {
    double itol = inner_tol, need = 0.5 * tol * nb / nr;
    if (need > itol) itol = need;
    float scale = (float)(1.0 / nr);
    for (i = 0; i < (long)n; ++i) { rl[i] = (float)(r[i] * (1.0 / nr)); xl[i] = 0; }
    (void)scale;
#pragma omp parallel for if (n > VO_OMP_MIN)
    for (i = 0; i < (long)n; ++i) zl[i] = rl[i] / dl[i];
    memcpy(pl, zl, sizeof(float) * n);
    float rz = 0;
    for (i = 0; i < (long)n; ++i) rz += rl[i] * zl[i];
    float rz0 = rz;
    for (vo_u32 it = 0; it < max_inner; ++it) {
      ++inner_total;
      vo_csr_spmv_s(n, rp, ci, vl, pl, 1.0f, 0.0f, tl);
      float alpha = rz / vo_dot_s(n, tl, pl);
      float rz_new = 0;
      for (i = 0; i < (long)n; ++i) {
        xl[i] += alpha * pl[i];
        rl[i] -= alpha * tl[i];
        zl[i] = rl[i] / dl[i];
        rz_new += rl[i] * zl[i];
      }
      if (fabs(rz_new / rz0) < itol * itol) break;
      float beta = rz_new / rz;
      rz = rz_new;
      for (i = 0; i < (long)n; ++i) pl[i] = zl[i] + beta * pl[i];
    }
    for (i = 0; i < (long)n; ++i) x[i] += nr * (double)xl[i];
    vo_csr_spmv_d(n, rp, ci, v, x, 1.0, 0.0, r);
    for (i = 0; i < (long)n; ++i) r[i] = b[i] - r[i];
    nr = sqrt(vo_dot_d(n, r, r));
    ++outer;
  }
  if (outer_out) *outer_out = outer;
  if (inner_total_out) *inner_total_out = inner_total;
  if (relres_out) *relres_out = nb > 0 ? nr / nb : 0;
  free(r); free(vl); free(dl); free(rl); free(zl); free(pl); free(tl); free(xl);
}

/* ------------------------------------------------------------------------ */
/* ILU0 -- detail/ilu/ilu0.hpp:77-140 (IKJ variant, Saad 1996)              */
/* ------------------------------------------------------------------------ */
void vo_ilu0_factor_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, double *lu) {
  for (vo_u32 i = 1; i < n; ++i) {
    vo_u32 ib = rp[i], ie = rp[i + 1];
    for (vo_u32 bk = ib; bk < ie; ++bk) {
      vo_u32 k = ci[bk];
      if (k >= i) continue;
      vo_u32 kb = rp[k], ke = rp[k + 1];
      double a_kk = 0;
      for (vo_u32 q = kb; q < ke; ++q)
        if (ci[q] == k) { a_kk = lu[q]; break; }
      lu[bk] /= a_kk;
      double a_ik = lu[bk];
      for (vo_u32 bj = ib; bj < ie; ++bj) {
        vo_u32 j = ci[bj];
        if (j <= k) continue;
        double a_kj = 0;
        for (vo_u32 q = kb; q < ke; ++q)
          if (ci[q] == j) { a_kj = lu[q]; break; }
        lu[bj] -= a_ik * a_kj;
      }
    }
  }
}

/* level_scheduling_setup_impl -- detail/ilu/common.hpp:50-187.  A row's
 * elimination level is one more than the largest level among the columns it
 * depends on; run e collects, for every row (ascending), the entries whose
 * column lies in level e. */
size_t vo_level_setup_d(vo_u32 n, const vo_u32 *rp, const vo_u32 *ci, const double *lu,
                        const double *udiag, int setup_U, size_t *total_rows, size_t *total_nnz,
                        vo_u32 *level_ptr, vo_u32 *row_index, vo_u32 *row_ptr, vo_u32 *cols,
                        double *vals) {
  vo_u32 *lev = (vo_u32 *)calloc(n ? n : 1, sizeof(vo_u32));
  vo_u32 maxlev = 0;
  for (vo_u32 r2 = 0; r2 < n; ++r2) {
    vo_u32 row = setup_U ? n - 1 - r2 : r2, e = 0;
    for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k) {
      vo_u32 c = ci[k];
      if ((!setup_U && c < row) || (setup_U && c > row))
        if (lev[c] > e) e = lev[c];
    }
    lev[row] = e + 1;
    if (e + 1 > maxlev) maxlev = e + 1;
  }
  /* count rows and entries per run */
  size_t *run_rows = (size_t *)calloc((size_t)maxlev + 2, sizeof(size_t));
  size_t *run_nnz = (size_t *)calloc((size_t)maxlev + 2, sizeof(size_t));
  vo_u32 *seen = (vo_u32 *)calloc((size_t)maxlev + 2, sizeof(vo_u32));
  for (vo_u32 row = 0; row < n; ++row) {
    for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k) {
      vo_u32 c = ci[k];
      if ((!setup_U && c < row) || (setup_U && c > row)) {
        vo_u32 e = lev[c];
        run_nnz[e] += 1;
        if (seen[e] != row + 1) { seen[e] = row + 1; run_rows[e] += 1; }
      }
    }
  }
  size_t nlev = 0, trows = 0, tnnz = 0;
  for (vo_u32 e = 1; e <= maxlev; ++e)
    if (run_rows[e] > 0) { ++nlev; trows += run_rows[e]; tnnz += run_nnz[e]; }
  if (total_rows) *total_rows = trows;
  if (total_nnz) *total_nnz = tnnz;
  if (level_ptr) {
    size_t L = 0, ro = 0, no = 0;
    level_ptr[0] = 0;
    row_ptr[0] = 0;
    for (vo_u32 e = 1; e <= maxlev; ++e) {
      if (run_rows[e] == 0) continue;
      for (vo_u32 row = 0; row < n; ++row) {
        int any = 0;
        for (vo_u32 k = rp[row]; k < rp[row + 1]; ++k) {
          vo_u32 c = ci[k];
          if (((!setup_U && c < row) || (setup_U && c > row)) && lev[c] == e) {
            cols[no] = c;
            vals[no] = setup_U ? lu[k] / udiag[row] : lu[k];
            ++no;
            any = 1;
          }
        }
        if (any) { row_index[ro] = row; ++ro; row_ptr[ro] = (vo_u32)no; }
      }
      level_ptr[++L] = (vo_u32)ro;
    }
  }
  free(lev); free(run_rows); free(run_nnz); free(seen);
  return nlev;
}

/* level_scheduling_substitute -- host_based/misc_operations.hpp:41-72 */
void vo_level_substitute_d(size_t nlev, const vo_u32 *level_ptr, const vo_u32 *row_index,
                           const vo_u32 *row_ptr, const vo_u32 *cols, const double *vals,
                           double *vec) {
  for (size_t L = 0; L < nlev; ++L) {
    long r0 = level_ptr[L], r1 = level_ptr[L + 1], r;
#pragma omp parallel for if (r1 - r0 > VO_OMP_MIN)
    for (r = r0; r < r1; ++r) {
      vo_u32 row = row_index[r];
      double s = vec[row];
      for (vo_u32 j = row_ptr[r]; j < row_ptr[r + 1]; ++j) s -= vec[cols[j]] * vals[j];
      vec[row] = s;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* CSR transpose with entry map (adjoint path; no reference counterpart).   */
/* ------------------------------------------------------------------------ */
void vo_csr_transpose_d(vo_u32 n_rows, vo_u32 n_cols, const vo_u32 *rp, const vo_u32 *ci,
                        const double *v, vo_u32 *trp, vo_u32 *tci, double *tv, vo_u32 *map) {
  memset(trp, 0, sizeof(vo_u32) * ((size_t)n_cols + 1));
  for (vo_u32 r = 0; r < n_rows; ++r)
    for (vo_u32 k = rp[r]; k < rp[r + 1]; ++k) trp[ci[k] + 1] += 1;
  for (vo_u32 c = 0; c < n_cols; ++c) trp[c + 1] += trp[c];
  vo_u32 *fill = (vo_u32 *)malloc(sizeof(vo_u32) * (n_cols ? n_cols : 1));
  memcpy(fill, trp, sizeof(vo_u32) * n_cols);
  for (vo_u32 r = 0; r < n_rows; ++r)
    for (vo_u32 k = rp[r]; k < rp[r + 1]; ++k) {
      vo_u32 pos = fill[ci[k]]++;
      tci[pos] = r;
      tv[pos] = v[k];
      map[pos] = k;
    }
  free(fill);
}
