// mixed.cu -- the two mixed-precision solvers.
//
// mixed_cg_solve: linalg::solve(A, b, mixed_precision_cg_tag) of
//   mixed_precision_cg.hpp:99-186 -- FP32 CG on an FP32 copy of A, restarted
//   from the FP64 residual b - A x whenever <r,r>_32 < inner_tol * <r0,r0>_32.
//
// refined_cg_solve: FP64 iterative refinement around FP32 Jacobi-PCG inner
//   solves (no reference counterpart).  Jacobi-PCG on A equals CG on the
//   symmetrically scaled matrix D^-1/2 A D^-1/2, so the inner solver is the
//   two-kernel pipelined CG on a cached FP32 copy of that matrix: FP32 values
//   and vectors halve the bytes of the memory-bound loop and no diagonal is
//   read per iteration.  When the matrix lies on at most 16 diagonals
//   (stencils) the copy is stored by diagonal (DIA, no column indices), which
//   halves the inner product's matrix bytes again.  FP64 is used only for
//   r = b - A x, x += d and ||r||.
#include <algorithm>
#include <cmath>

#include "formats.hpp"
#include "vecpass.cuh"

namespace vclgb {

template <typename T>
void cg_solve(Backend &, Matrix &, const T *, T *, vclgbSolverTag *, const Precond *);

struct McSt {
  double nrhs2, new_ip, error, tol;
  float inner_ip, initial, alpha, beta, inner_tol;
  unsigned iters, max_iters;
  int done;
  int restart_skip;
};

struct McInit {
  static constexpr int NDOT = 1;
  const double *b; double *x, *res; float *p, *r, *xl; McSt *st;
  struct S {};
  __device__ bool skip() const { return false; }
  __device__ S load() const { return {}; }
  __device__ void apply(size_t i, S, double (&d)[1]) const {
    double bi = b[i];
    x[i] = 0.0;
    res[i] = bi;
    float pf = (float)bi;
    p[i] = pf;
    r[i] = pf;
    xl[i] = 0.f;
    d[0] += bi * bi;
  }
  __device__ void finalize(const double (&s)[1]) const {
    st->nrhs2 = s[0];
    st->new_ip = 0;
    st->error = 0;
    st->iters = 0;
    st->inner_ip = (float)s[0];
    st->initial = (float)s[0];
    st->restart_skip = 1;
    st->done = s[0] <= 0 ? kConverged : (st->max_iters == 0 ? kMaxIters : kRunning);
  }
};

struct EpiMc1 {  // tmp = A32 p; alpha = inner_ip / <tmp,p>
  static constexpr int NDOT = 1;
  float *tmp; const float *p; McSt *st;
  struct Pre { float p; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ Pre pre(uint32_t r) const { return {p[r]}; }
  __device__ void row(uint32_t r, float acc, const Pre &v, float (&d)[1]) const {
    tmp[r] = acc;
    d[0] += acc * v.p;
  }
  __device__ void finalize(const float (&s)[1]) const {
    st->iters += 1;
    st->alpha = st->inner_ip / s[0];
  }
};

struct McUpd {  // x32 += a p; r32 -= a tmp; <r32,r32>; restart test
  static constexpr int NDOT = 1;
  float *xl, *r; const float *p, *tmp; McSt *st;
  struct S { float a; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->alpha}; }
  __device__ void apply(size_t i, S c, float (&d)[1]) const {
    xl[i] += c.a * p[i];
    float v = r[i] - c.a * tmp[i];
    r[i] = v;
    d[0] += v * v;
  }
  __device__ void finalize(const float (&s)[1]) const {
    float nw = s[0];
    st->beta = nw / st->inner_ip;
    st->inner_ip = nw;
    bool restart = nw < st->inner_tol * st->initial || st->iters == st->max_iters;
    st->restart_skip = restart ? 0 : 1;
  }
};

struct McP {  // p = r32 + beta p
  static constexpr int NDOT = 0;
  float *p; const float *r; McSt *st;
  struct S { float b; };
  __device__ bool skip() const { return st->done != kRunning; }
  __device__ S load() const { return {st->beta}; }
  __device__ void apply(size_t i, S c, float (&)[1]) const { p[i] = r[i] + c.b * p[i]; }
  __device__ void finalize(const float (&)[1]) const {}
};

struct McAddX {  // x += x32
  static constexpr int NDOT = 0;
  double *x; const float *xl; McSt *st;
  struct S {};
  __device__ bool skip() const { return st->restart_skip != 0; }
  __device__ S load() const { return {}; }
  __device__ void apply(size_t i, S, double (&)[1]) const { x[i] += (double)xl[i]; }
  __device__ void finalize(const double (&)[1]) const {}
};

struct EpiMcRes {  // res = b - A x (FP64); <res,res>; outer test
  static constexpr int NDOT = 1;
  double *res; const double *b; McSt *st;
  struct Pre { double b; };
  __device__ bool skip() const { return st->restart_skip != 0; }
  __device__ Pre pre(uint32_t r) const { return {b[r]}; }
  __device__ void row(uint32_t r, double acc, const Pre &pv, double (&d)[1]) const {
    double v = pv.b - acc;
    res[r] = v;
    d[0] += v * v;
  }
  __device__ void finalize(const double (&s)[1]) const {
    st->new_ip = s[0];
    st->error = sqrt(s[0] / st->nrhs2);
    if (s[0] / st->nrhs2 < st->tol * st->tol) {
      st->done = kConverged;
      st->restart_skip = 1;
    } else if (st->iters >= st->max_iters) {
      st->done = kMaxIters;
      st->restart_skip = 1;
    }
  }
};

struct McReset {  // p32 = res; x32 = 0; r32 = p32
  static constexpr int NDOT = 0;
  float *p, *r, *xl; const double *res; McSt *st;
  struct S {};
  __device__ bool skip() const { return st->restart_skip != 0; }
  __device__ S load() const { return {}; }
  __device__ void apply(size_t i, S, float (&)[1]) const {
    float v = (float)res[i];
    p[i] = v;
    r[i] = v;
    xl[i] = 0.f;
  }
  __device__ void finalize(const float (&)[1]) const {}
};

struct McResetScalars {
  McSt *st;
  __device__ void operator()() const {
    if (st->restart_skip) return;
    st->initial = (float)st->new_ip;
    st->inner_ip = (float)st->new_ip;
    st->restart_skip = 1;
  }
};

static Matrix &f32_copy(Backend &be, Matrix &A) {
  if (!A.f32_copy) A.f32_copy = convert_f32(be, A);
  return *A.f32_copy;
}

void mixed_cg_solve(Backend &be, Matrix &A, const double *b, double *x, vclgbSolverTag *tag,
                    float inner_tol) {
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "CG needs a square matrix");
  require(A.format == VCLGB_CSR, VCLGB_UNSUPPORTED, "mixed CG runs on CSR matrices");
  const uint32_t n = A.rows;
  Matrix &A32 = f32_copy(be, A);
  DevBuf stb(sizeof(McSt), be.stream), part(8 * kMaxSpmvGrid * sizeof(double), be.stream),
      cnt(64, be.stream);
  size_t n1 = std::max<size_t>(n, 1);
  DevBuf res(n1 * 8, be.stream), p(n1 * 4, be.stream), r(n1 * 4, be.stream),
      xl(n1 * 4, be.stream), tmp(n1 * 4, be.stream);
  McSt h;
  std::memset(&h, 0, sizeof(h));
  h.tol = tag->tol;
  h.inner_tol = inner_tol;
  h.max_iters = tag->max_iters;
  VCLGB_CUDA(cudaMemcpyAsync(stb.ptr, &h, sizeof(h), cudaMemcpyHostToDevice, be.stream));
  VCLGB_CUDA(cudaMemsetAsync(cnt.ptr, 0, 64, be.stream));
  McSt *st = stb.as<McSt>();
  Reduction red{part.ptr, cnt.as<unsigned>()};
  vec_pass<double>(be, n, McInit{b, x, res.as<double>(), p.as<float>(), r.as<float>(),
                                 xl.as<float>(), st}, red);
  const int *done = &st->done;
  uint32_t every = tag->check_every ? tag->check_every : 16;
  run_iterations(be, done, tag->max_iters / every + 2, every, true, [&]() {
    spmv_launch<float>(be, A32, p.as<float>(), 0, 1, EpiMc1{tmp.as<float>(), p.as<float>(), st},
                       red);
    vec_pass<float>(be, n, McUpd{xl.as<float>(), r.as<float>(), p.as<float>(), tmp.as<float>(), st}, red);
    vec_pass<float>(be, n, McP{p.as<float>(), r.as<float>(), st}, red);
    vec_pass<double>(be, n, McAddX{x, xl.as<float>(), st}, red);
    spmv_launch<double>(be, A, x, 0, 1, EpiMcRes{res.as<double>(), b, st}, red);
    vec_pass<float>(be, n, McReset{p.as<float>(), r.as<float>(), xl.as<float>(), res.as<double>(), st}, red);
    scalar_step(be, McResetScalars{st});
  });
  VCLGB_CUDA(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  tag->iters = h.iters;
  tag->error = h.error;
  tag->status = h.done == kConverged ? VCLGB_SUCCESS
              : h.done == kMaxIters  ? VCLGB_NOT_CONVERGED
                                     : VCLGB_BREAKDOWN;
}

// ---------------------------------------------------------------------------
// refined CG
// ---------------------------------------------------------------------------
__global__ void inv_sqrt_diag_kernel(uint32_t n, const double *__restrict__ d, double *dis,
                                     unsigned *bad) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    double v = d[i];
    if (!(v > 0.0)) atomicOr(bad, 1u);
    dis[i] = v > 0.0 ? 1.0 / sqrt(v) : 0.0;
  }
}

__global__ void scale_values_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                    const uint32_t *__restrict__ ci, const double *__restrict__ v,
                                    const double *__restrict__ dis, float *out) {
  for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < rows;
       r += (size_t)gridDim.x * blockDim.x) {
    double dr = dis[r];
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k) out[k] = (float)(v[k] * dr * dis[ci[k]]);
  }
}

static Matrix &f32_scaled(Backend &be, Matrix &A) {
  if (A.f32_scaled) return *A.f32_scaled;
  DevBuf d;
  extract_diag(be, A, d, false);
  A.inv_sqrt_diag.alloc(std::max<size_t>(A.rows, 1) * 8, be.stream);
  DevBuf bad(4, be.stream);
  VCLGB_CUDA(cudaMemsetAsync(bad.ptr, 0, 4, be.stream));
  int g = waves_grid(be, 256, 8, A.rows);
  inv_sqrt_diag_kernel<<<g, 256, 0, be.stream>>>(A.rows, d.as<double>(),
                                                 A.inv_sqrt_diag.as<double>(), bad.as<unsigned>());
  be.launches++;
  unsigned hb = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&hb, bad.ptr, 4, cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  require(hb == 0, VCLGB_ZERO_ON_DIAGONAL, "refined CG needs a positive diagonal");
  auto m = std::make_unique<Matrix>();
  m->format = VCLGB_CSR;
  m->prec = VCLGB_FLOAT32;
  m->rows = A.rows;
  m->cols = A.cols;
  m->nnz = A.nnz;
  m->row_ptr = A.row_ptr;
  m->col_idx = A.col_idx;
  m->own_values.alloc(std::max<uint64_t>(A.nnz, 1) * 4, be.stream);
  scale_values_kernel<<<g, 256, 0, be.stream>>>(A.rows, A.row_ptr, A.col_idx,
                                                static_cast<const double *>(A.values),
                                                A.inv_sqrt_diag.as<double>(),
                                                m->own_values.as<float>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  m->values = m->own_values.ptr;
  m->num_bins = A.num_bins;
  for (int i = 0; i < A.num_bins; ++i) m->bins[i] = A.bins[i];
  m->max_row_len = A.max_row_len;
  A.f32_scaled = std::move(m);
  return *A.f32_scaled;
}

struct IrInit {  // x = 0; r = b; ||b||^2
  static constexpr int NDOT = 1;
  const double *b; double *x, *r, *out;
  struct S {};
  __device__ bool skip() const { return false; }
  __device__ S load() const { return {}; }
  __device__ void apply(size_t i, S, double (&d)[1]) const {
    double v = b[i];
    x[i] = 0.0;
    r[i] = v;
    d[0] += v * v;
  }
  __device__ void finalize(const double (&s)[1]) const { *out = s[0]; }
};

struct IrRhs {  // rhat = D^-1/2 r / ||r|| in FP32
  static constexpr int NDOT = 0;
  float *rh; const double *r, *dis; double inv_nr;
  struct S {};
  __device__ bool skip() const { return false; }
  __device__ S load() const { return {}; }
  __device__ void apply(size_t i, S, double (&)[1]) const {
    rh[i] = (float)(dis[i] * r[i] * inv_nr);
  }
  __device__ void finalize(const double (&)[1]) const {}
};

struct IrUpdate {  // x += ||r|| D^-1/2 y
  static constexpr int NDOT = 0;
  double *x; const float *y; const double *dis; double nr;
  struct S {};
  __device__ bool skip() const { return false; }
  __device__ S load() const { return {}; }
  __device__ void apply(size_t i, S, double (&)[1]) const { x[i] += nr * dis[i] * (double)y[i]; }
  __device__ void finalize(const double (&)[1]) const {}
};

struct EpiIrResid {  // r = b - A x; ||r||^2
  static constexpr int NDOT = 1;
  double *r; const double *b; double *out;
  struct Pre { double b; };
  __device__ bool skip() const { return false; }
  __device__ Pre pre(uint32_t i) const { return {b[i]}; }
  __device__ void row(uint32_t i, double acc, const Pre &pv, double (&d)[1]) const {
    double v = pv.b - acc;
    r[i] = v;
    d[0] += v * v;
  }
  __device__ void finalize(const double (&s)[1]) const { *out = s[0]; }
};

void refined_cg_solve(Backend &be, Matrix &A, const double *b, double *x, vclgbSolverTag *tag,
                      double inner_tol, uint32_t max_outer, uint32_t *outer_out) {
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "CG needs a square matrix");
  require(A.format == VCLGB_CSR, VCLGB_UNSUPPORTED, "refined CG runs on CSR matrices");
  const uint32_t n = A.rows;
  if (inner_tol <= 0) inner_tol = 1e-4;
  if (max_outer == 0) max_outer = 30;
  Matrix &Ah = f32_scaled(be, A);
  // a banded matrix (stencil) runs its inner iterations on the DIA form of the
  // scaled copy: no column indices, 4 bytes per stored slot
  if (!A.f32_scaled_dia_tried) {
    A.f32_scaled_dia = try_convert_dia(be, Ah, 1.25);
    A.f32_scaled_dia_tried = true;
  }
  Matrix *Ad = A.f32_scaled_dia.get();
  size_t n1 = std::max<size_t>(n, 1);
  DevBuf r(n1 * 8, be.stream), rh(n1 * 4, be.stream), y(n1 * 4, be.stream),
      part(8 * kMaxSpmvGrid * 8, be.stream), cnt(64, be.stream), sc(16, be.stream);
  VCLGB_CUDA(cudaMemsetAsync(cnt.ptr, 0, 64, be.stream));
  Reduction red{part.ptr, cnt.as<unsigned>()};
  double *d_sc = sc.as<double>();
  vec_pass<double>(be, n, IrInit{b, x, r.as<double>(), d_sc}, red);
  double bb = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&bb, d_sc, 8, cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  const double nb = std::sqrt(bb);
  double nr = nb;
  uint32_t outer = 0, inner_total = 0;
  vclgbStatus status = VCLGB_SUCCESS;
  while (nb > 0 && nr / nb >= tag->tol) {
    if (outer >= max_outer || inner_total >= tag->max_iters) {
      status = VCLGB_NOT_CONVERGED;
      break;
    }
    double itol = std::max(inner_tol, 0.5 * tag->tol * nb / nr);
    vec_pass<double>(be, n, IrRhs{rh.as<float>(), r.as<double>(), A.inv_sqrt_diag.as<double>(),
                                  1.0 / nr}, red);
    vclgbSolverTag it;
    std::memset(&it, 0, sizeof(it));
    it.tol = itol;
    it.max_iters = tag->max_iters - inner_total;
    it.check_every = tag->check_every;
    cg_solve<float>(be, Ad ? *Ad : Ah, rh.as<float>(), y.as<float>(), &it, nullptr);
    inner_total += it.iters;
    vec_pass<double>(be, n, IrUpdate{x, y.as<float>(), A.inv_sqrt_diag.as<double>(), nr}, red);
    spmv_launch<double>(be, A, x, 0, 1, EpiIrResid{r.as<double>(), b, d_sc}, red);
    double rr = 0;
    VCLGB_CUDA(cudaMemcpyAsync(&rr, d_sc, 8, cudaMemcpyDeviceToHost, be.stream));
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    nr = std::sqrt(rr);
    ++outer;
    if (!std::isfinite(nr)) {
      status = VCLGB_BREAKDOWN;
      break;
    }
  }
  tag->iters = inner_total;
  tag->error = nb > 0 ? nr / nb : 0.0;
  tag->status = status;
  if (outer_out) *outer_out = outer;
}

}  // namespace vclgb
