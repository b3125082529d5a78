// batched.cu -- thousands of independent sparse systems solved in one
// persistent launch (no reference counterpart; the per-system algorithms are
// the reference's pipelined CG, cg.hpp:128-187, and pipelined BiCGStab,
// bicgstab.hpp:96-215, with the same stopping tests).
//
// The systems are the diagonal blocks of one block-diagonal CSR matrix.  A
// persistent grid pulls systems from a device work queue (largest first):
// the CTA that takes a system runs every iteration of it with block-level
// reductions only -- there is no grid-wide barrier, no device-side wait and no
// host round trip per iteration, and each system stops on its own
// convergence test (the per-system status array is the convergence mask).
// An autotuner picks the block size and lanes per row on a sample of the
// batch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>

#include "formats.hpp"
#include "vecpass.cuh"

namespace vclgb {

struct Batch {
  uint32_t nsys = 0;
  std::vector<uint32_t> h_sys_ptr;
  std::vector<int32_t> h_methods;
  DevBuf sys_ptr, methods, order, queue, iters, status, error;
  DevBuf ws;          // r, p, Ap, r0, s, As  (each sum(n) long)
  int block = 256, lanes = 2;
  bool tuned = false;
  const Matrix *A = nullptr;
};

// Block reduction of NV values whose sums thread 0 turns into the step's NS
// scalars: a butterfly per warp, warp 0 adds the warp sums, thread 0 runs
// step(sums, out) once and every thread reads out[] after the barrier.  Every
// thread re-adding the warp sums and repeating the step's divisions and
// square roots cost each iteration more FP64 work than the rows of a small
// system (GB300's FP64 pipe is narrow).  Deterministic: fixed order.
// red holds 4 * (BS / 32) + 8 values.
template <int BS, int NV, int NS, typename T, class F>
__device__ __forceinline__ void cta_step(T (&v)[NV], T *red, T (&out)[NS], F &&step) {
  constexpr int NW = BS / 32, P = Pow2<NV>::v, SPAN = 32 / P;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T w = warp_sum_multi<NV>(v, lane);
  __syncthreads();  // the previous step's readers are done with red[]
  if ((lane & (SPAN - 1)) == 0 && lane / SPAN < NV) red[(lane / SPAN) * NW + warp] = w;
  __syncthreads();
  if (warp == 0) {
    T t[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) t[i] = lane < NW ? red[i * NW + lane] : T(0);
    const T sum = warp_sum_multi<NV>(t, lane);
    T sums[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) sums[i] = __shfl_sync(0xffffffffu, sum, i * SPAN);
    if (lane == 0) {
      T o[NS];
      step(sums, o);
#pragma unroll
      for (int j = 0; j < NS; ++j) red[4 * NW + j] = o[j];
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NS; ++j) out[j] = red[4 * NW + j];
}

// y = A_k x on the rows [r0, r0+n) of system k; optional fused dots
template <int BS, int LANES, typename T, class F>
__device__ __forceinline__ void cta_spmv(const uint32_t *__restrict__ rp,
                                         const uint32_t *__restrict__ ci,
                                         const T *__restrict__ v, uint32_t r0, uint32_t n,
                                         const T *x, F &&on_row) {
  constexpr int GPW = 32 / LANES;
  const int lane = threadIdx.x & (LANES - 1);
  const int gw = (threadIdx.x & 31) / LANES;
  const int warp = threadIdx.x >> 5;
  constexpr int NW = BS / 32;
  for (uint32_t base = warp * GPW; base < n; base += NW * GPW) {
    uint32_t row = base + gw;
    T acc = 0;
    if (row < n) {
      uint32_t e = rp[r0 + row + 1];
      for (uint32_t k = rp[r0 + row] + lane; k < e; k += LANES) acc += v[k] * x[ci[k]];
    }
    acc = group_sum<LANES>(acc);
    if (lane == 0 && row < n) on_row(r0 + row, acc);
  }
}

template <typename T>
struct BatchArgs {
  const uint32_t *rp, *ci;
  const T *v;
  const uint32_t *sys_ptr;
  const int32_t *methods;
  const uint32_t *order;
  uint32_t nsys;
  unsigned *queue;
  const T *b;
  T *x, *r, *p, *Ap, *r0, *s, *As;
  double tol;
  uint32_t max_iters;
  uint32_t *iters;
  int32_t *status;
  double *error;
};

template <int BS, int LANES, typename T>
__global__ void __launch_bounds__(BS) batched_kernel(BatchArgs<T> a) {
  __shared__ T red[4 * (BS / 32) + 8];
  __shared__ uint32_t sys_sh;
  const double tol2 = a.tol * a.tol;
  constexpr T kGo = T(0), kStop = T(1), kBreak = T(2);  // step verdicts
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) sys_sh = atomicAdd(a.queue, 1u);
    __syncthreads();
    const uint32_t q = sys_sh;
    if (q >= a.nsys) return;
    const uint32_t k = a.order[q];
    const uint32_t r0 = a.sys_ptr[k], n = a.sys_ptr[k + 1] - r0;
    const int method = a.methods[k];
    T *x = a.x, *r = a.r, *p = a.p, *Ap = a.Ap;
    const T *b = a.b;
    uint32_t it = 0;
    int st = kMaxIters;
    double err = 0;   // thread 0's
    if (method == 0) {
      // ---- pipelined CG (cg.hpp:128-187) ----
      T d[1] = {0};
      for (uint32_t i = threadIdx.x; i < n; i += BS) {
        T bi = b[r0 + i];
        x[r0 + i] = 0; r[r0 + i] = bi; p[r0 + i] = bi;
        d[0] += bi * bi;
      }
      T nrhs2 = 0, rr = 0;  // thread 0's
      T o1[1];
      cta_step<BS>(d, red, o1, [&](const T (&sm)[1], T (&o)[1]) {
        const T nrm = sqrt(sm[0]);
        nrhs2 = nrm * nrm;  // norm_2(residual)^2 as cg.hpp:149
        rr = nrhs2;
        o[0] = nrhs2 <= T(0) ? kStop : kGo;
      });
      if (o1[0] != kGo) { st = kConverged; goto done; }
      {
        T e2[2] = {0, 0};
        cta_spmv<BS, LANES>(a.rp, a.ci, a.v, r0, n, p, [&](uint32_t row, T acc) {
          Ap[row] = acc; e2[0] += acc * acc; e2[1] += p[row] * acc;
        });
        T ab[2];
        cta_step<BS>(e2, red, ab, [&](const T (&sm)[2], T (&o)[2]) {
          const T alpha = rr / sm[1];
          const T nap = sqrt(sm[0]);
          o[0] = alpha;
          o[1] = (alpha * alpha * nap * nap - rr) / rr;
        });
        for (it = 1; it <= a.max_iters; ++it) {
          const T alpha = ab[0], beta = ab[1];
          T d1[1] = {0};
          for (uint32_t i = threadIdx.x; i < n; i += BS) {
            uint32_t g = r0 + i;
            T vp = p[g], vr = r[g];
            x[g] += alpha * vp;
            vr -= alpha * Ap[g];
            vp = vr + beta * vp;
            d1[0] += vr * vr;
            p[g] = vp; r[g] = vr;
          }
          T o0[1];
          // also orders the p writes before the SpMV reads
          cta_step<BS>(d1, red, o0, [&](const T (&sm)[1], T (&o)[1]) { rr = sm[0]; o[0] = 0; });
          T e[2] = {0, 0};
          cta_spmv<BS, LANES>(a.rp, a.ci, a.v, r0, n, p, [&](uint32_t row, T acc) {
            Ap[row] = acc; e[0] += acc * acc; e[1] += p[row] * acc;
          });
          T ov[3];
          cta_step<BS>(e, red, ov, [&](const T (&sm)[2], T (&o)[3]) {
            err = sqrt(fabs((double)rr) / (double)nrhs2);
            if (fabs((double)rr / (double)nrhs2) < tol2) { o[2] = kStop; return; }
            const T al = rr / sm[1];
            const T be = (al * al * sm[0] - rr) / rr;
            o[0] = al;
            o[1] = be;
            o[2] = (!isfinite(al) || !isfinite(be)) ? kBreak : kGo;
          });
          if (ov[2] == kStop) { st = kConverged; break; }
          if (ov[2] == kBreak) { st = kBreakdown; break; }
          ab[0] = ov[0];
          ab[1] = ov[1];
        }
        if (it > a.max_iters) it = a.max_iters;
      }
    } else {
      // ---- pipelined BiCGStab (bicgstab.hpp:96-215) ----
      T *rs = a.r0, *s = a.s, *As = a.As;
      T d[1] = {0};
      for (uint32_t i = threadIdx.x; i < n; i += BS) {
        uint32_t g = r0 + i;
        T bi = b[g];
        x[g] = 0; r[g] = bi; p[g] = bi; rs[g] = bi;
        d[0] += bi * bi;
      }
      T nrhs = 0, r_r0 = 0, Ap_r0 = 0, s_s = 0;  // thread 0's
      T o1[1];
      cta_step<BS>(d, red, o1, [&](const T (&sm)[1], T (&o)[1]) {
        nrhs = sqrt(sm[0]);
        r_r0 = nrhs * nrhs;
        o[0] = nrhs <= T(0) ? kStop : kGo;
      });
      if (o1[0] != kGo) { st = kConverged; goto done; }
      for (it = 1; it <= a.max_iters; ++it) {
        T e1[1] = {0};
        cta_spmv<BS, LANES>(a.rp, a.ci, a.v, r0, n, p, [&](uint32_t row, T acc) {
          Ap[row] = acc; e1[0] += acc * rs[row];
        });
        T oa[1];
        cta_step<BS>(e1, red, oa, [&](const T (&sm)[1], T (&o)[1]) {
          Ap_r0 = sm[0];
          o[0] = r_r0 / Ap_r0;
        });
        const T alpha = oa[0];
        T e2[1] = {0};
        for (uint32_t i = threadIdx.x; i < n; i += BS) {
          uint32_t g = r0 + i;
          T vs = r[g] - alpha * Ap[g];
          s[g] = vs;
          e2[0] += vs * vs;
        }
        T os[1];
        cta_step<BS>(e2, red, os, [&](const T (&sm)[1], T (&o)[1]) { s_s = sm[0]; o[0] = 0; });
        T e3[3] = {0, 0, 0};
        cta_spmv<BS, LANES>(a.rp, a.ci, a.v, r0, n, s, [&](uint32_t row, T acc) {
          As[row] = acc; e3[0] += acc * acc; e3[1] += s[row] * acc; e3[2] += acc * rs[row];
        });
        T ow[3];
        cta_step<BS>(e3, red, ow, [&](const T (&sm)[3], T (&o)[3]) {
          const T be = -sm[2] / Ap_r0;
          const T om = sm[1] / sm[0];
          const T rn = sqrt(s_s - T(2) * om * sm[1] + om * om * sm[0]);
          err = (double)rn / (double)nrhs;
          o[0] = be;
          o[1] = om;
          if (err < a.tol) o[2] = kStop;
          else if (!isfinite(o[1]) || !isfinite(be) || !isfinite(r_r0 / Ap_r0)) o[2] = kBreak;
          else o[2] = kGo;
        });
        if (ow[2] == kStop) { st = kConverged; break; }
        if (ow[2] == kBreak) { st = kBreakdown; break; }
        const T beta = ow[0], omega = ow[1];
        T e4[1] = {0};
        for (uint32_t i = threadIdx.x; i < n; i += BS) {
          uint32_t g = r0 + i;
          T vp = p[g], vs = s[g];
          x[g] += alpha * vp + omega * vs;
          T vr = vs - omega * As[g];
          vp = vr + beta * (vp - omega * Ap[g]);
          e4[0] += vr * rs[g];
          r[g] = vr;
          p[g] = vp;
        }
        T orr[1];
        cta_step<BS>(e4, red, orr, [&](const T (&sm)[1], T (&o)[1]) { r_r0 = sm[0]; o[0] = 0; });
      }
      if (it > a.max_iters) it = a.max_iters;
    }
  done:
    if (threadIdx.x == 0) {
      a.iters[k] = it;
      a.status[k] = st;
      a.error[k] = err;
    }
  }
}

__global__ void batch_check_kernel(const uint32_t *__restrict__ rp, const uint32_t *__restrict__ ci,
                                   const uint32_t *__restrict__ sys_ptr, uint32_t nsys,
                                   unsigned *bad) {
  // every entry of system k must stay inside its diagonal block
  for (size_t k = blockIdx.x; k < nsys; k += gridDim.x) {
    uint32_t r0 = sys_ptr[k], r1 = sys_ptr[k + 1];
    for (uint32_t j = rp[r0] + threadIdx.x; j < rp[r1]; j += blockDim.x)
      if (ci[j] < r0 || ci[j] >= r1) atomicOr(bad, 1u);
  }
}

using BatchKernel = void (*)(BatchArgs<double>);

static BatchKernel pick(int block, int lanes) {
#define VCLGB_BK(BS, L) if (block == BS && lanes == L) return batched_kernel<BS, L, double>
  VCLGB_BK(128, 1); VCLGB_BK(128, 2); VCLGB_BK(128, 4); VCLGB_BK(128, 8);
  VCLGB_BK(256, 1); VCLGB_BK(256, 2); VCLGB_BK(256, 4); VCLGB_BK(256, 8);
  VCLGB_BK(512, 1); VCLGB_BK(512, 2); VCLGB_BK(512, 4); VCLGB_BK(512, 8);
#undef VCLGB_BK
  return nullptr;
}

static void launch(Backend &be, Batch &bt, const double *b, double *x, double tol,
                   uint32_t max_iters, uint32_t nsys_limit) {
  BatchKernel kern = pick(bt.block, bt.lanes);
  require(kern != nullptr, VCLGB_INVALID_ARGUMENT, "unsupported batch configuration");
  size_t N = bt.h_sys_ptr.back();
  double *w = bt.ws.as<double>();
  BatchArgs<double> a;
  a.rp = bt.A->row_ptr;
  a.ci = bt.A->col_idx;
  a.v = static_cast<const double *>(bt.A->values);
  a.sys_ptr = bt.sys_ptr.as<uint32_t>();
  a.methods = bt.methods.as<int32_t>();
  a.order = bt.order.as<uint32_t>();
  a.nsys = std::min(bt.nsys, nsys_limit);
  a.queue = bt.queue.as<unsigned>();
  a.b = b;
  a.x = x;
  a.r = w; a.p = w + N; a.Ap = w + 2 * N; a.r0 = w + 3 * N; a.s = w + 4 * N; a.As = w + 5 * N;
  a.tol = tol;
  a.max_iters = max_iters;
  a.iters = bt.iters.as<uint32_t>();
  a.status = bt.status.as<int32_t>();
  a.error = bt.error.as<double>();
  int per_sm = 0;
  VCLGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, bt.block, 0));
  int grid = std::max(1, per_sm) * be.num_sms;
  grid = (int)std::min<uint64_t>((uint64_t)grid, std::max<uint32_t>(a.nsys, 1));
  VCLGB_CUDA(cudaMemsetAsync(bt.queue.ptr, 0, sizeof(unsigned), be.stream));
  kern<<<grid, bt.block, 0, be.stream>>>(a);
  be.launches++;
  VCLGB_CHECK_LAUNCH();
}

Batch *batch_create(Backend &be, const Matrix &A, uint32_t nsys, const uint32_t *h_sys_ptr,
                    const int32_t *h_methods) {
  require(A.format == VCLGB_CSR && A.prec == VCLGB_FLOAT64, VCLGB_INVALID_ARGUMENT,
          "batched systems are given as one FP64 block-diagonal CSR matrix");
  require(nsys > 0 && h_sys_ptr && h_methods, VCLGB_INVALID_ARGUMENT, "empty batch");
  require(h_sys_ptr[0] == 0 && h_sys_ptr[nsys] == A.rows, VCLGB_INVALID_ARGUMENT,
          "system offsets must cover the matrix rows");
  auto bt = std::make_unique<Batch>();
  bt->nsys = nsys;
  bt->A = &A;
  bt->h_sys_ptr.assign(h_sys_ptr, h_sys_ptr + nsys + 1);
  bt->h_methods.assign(h_methods, h_methods + nsys);
  for (uint32_t k = 0; k < nsys; ++k) {
    require(h_sys_ptr[k + 1] >= h_sys_ptr[k], VCLGB_INVALID_ARGUMENT, "system offsets decrease");
    require(h_methods[k] == 0 || h_methods[k] == 1, VCLGB_INVALID_ARGUMENT,
            "method must be 0 (CG) or 1 (BiCGStab)");
  }
  // work queue order: largest systems first (longest-processing-time rule)
  std::vector<uint32_t> order(nsys);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    return h_sys_ptr[a + 1] - h_sys_ptr[a] > h_sys_ptr[b + 1] - h_sys_ptr[b];
  });
  auto up = [&](DevBuf &d, const void *src, size_t bytes) {
    d.alloc(std::max<size_t>(bytes, 4), be.stream);
    VCLGB_CUDA(cudaMemcpyAsync(d.ptr, src, bytes, cudaMemcpyHostToDevice, be.stream));
  };
  up(bt->sys_ptr, h_sys_ptr, (nsys + 1) * 4);
  up(bt->methods, h_methods, nsys * 4);
  up(bt->order, order.data(), nsys * 4);
  bt->queue.alloc(64, be.stream);
  bt->iters.alloc(nsys * 4, be.stream);
  bt->status.alloc(nsys * 4, be.stream);
  bt->error.alloc(nsys * 8, be.stream);
  bt->ws.alloc(std::max<size_t>((size_t)A.rows, 1) * 6 * sizeof(double), be.stream);
  DevBuf bad(4, be.stream);
  VCLGB_CUDA(cudaMemsetAsync(bad.ptr, 0, 4, be.stream));
  batch_check_kernel<<<std::min<uint32_t>(nsys, 4096), 256, 0, be.stream>>>(
      A.row_ptr, A.col_idx, bt->sys_ptr.as<uint32_t>(), nsys, bad.as<unsigned>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  unsigned hb = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&hb, bad.ptr, 4, cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  require(hb == 0, VCLGB_INVALID_MATRIX, "an entry couples two systems (matrix not block-diagonal)");
  // default configuration from the mean system size until tuned
  double mean_n = (double)A.rows / nsys, mean_len = A.rows ? (double)A.nnz / A.rows : 1.0;
  bt->block = mean_n > 8192 ? 512 : 256;
  bt->lanes = mean_len > 12 ? 8 : (mean_len > 6 ? 4 : 2);
  return bt.release();
}

// Autotuner: times every (block size, lanes per row) pair on a sample of the
// batch -- every 8th system of the size-sorted order, so the sample spans the
// size range -- with a fixed iteration cap, and keeps the fastest.
void batch_tune(Backend &be, Batch &bt, const double *b) {
  const int blocks[] = {128, 256, 512};
  const int lanes[] = {1, 2, 4, 8};
  DevBuf xs(std::max<size_t>(bt.h_sys_ptr.back(), 1) * 8, be.stream);
  // sample: reorder the queue so the first nsample entries are every 8th system
  std::vector<uint32_t> order(bt.nsys);
  VCLGB_CUDA(cudaMemcpyAsync(order.data(), bt.order.ptr, bt.nsys * 4, cudaMemcpyDeviceToHost,
                             be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  std::vector<uint32_t> sample;
  for (uint32_t i = 0; i < bt.nsys; i += 8) sample.push_back(order[i]);
  DevBuf saved(std::move(bt.order));
  bt.order.alloc(sample.size() * 4, be.stream);
  VCLGB_CUDA(cudaMemcpyAsync(bt.order.ptr, sample.data(), sample.size() * 4,
                             cudaMemcpyHostToDevice, be.stream));
  cudaEvent_t e0, e1;
  VCLGB_CUDA(cudaEventCreate(&e0));
  VCLGB_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int bb = bt.block, bl = bt.lanes;
  for (int B : blocks)
    for (int L : lanes) {
      bt.block = B;
      bt.lanes = L;
      launch(be, bt, b, xs.as<double>(), 0.0, 40, (uint32_t)sample.size());  // warm
      VCLGB_CUDA(cudaEventRecord(e0, be.stream));
      launch(be, bt, b, xs.as<double>(), 0.0, 40, (uint32_t)sample.size());
      VCLGB_CUDA(cudaEventRecord(e1, be.stream));
      VCLGB_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      VCLGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) { best = ms; bb = B; bl = L; }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  bt.block = bb;
  bt.lanes = bl;
  bt.order = std::move(saved);
  bt.tuned = true;
}

// returns true when every system converged
bool batch_solve(Backend &be, Batch &bt, const double *b, double *x, double tol,
                 uint32_t max_iters, uint32_t *h_iters, int32_t *h_status, double *h_error) {
  launch(be, bt, b, x, tol, max_iters, bt.nsys);
  std::vector<int32_t> st(bt.nsys);
  if (h_iters)
    VCLGB_CUDA(cudaMemcpyAsync(h_iters, bt.iters.ptr, bt.nsys * 4, cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaMemcpyAsync(st.data(), bt.status.ptr, bt.nsys * 4, cudaMemcpyDeviceToHost, be.stream));
  if (h_error)
    VCLGB_CUDA(cudaMemcpyAsync(h_error, bt.error.ptr, bt.nsys * 8, cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  bool all = true;
  for (uint32_t k = 0; k < bt.nsys; ++k) {
    int32_t s = st[k] == kConverged ? VCLGB_SUCCESS
              : st[k] == kMaxIters  ? VCLGB_NOT_CONVERGED
                                    : VCLGB_BREAKDOWN;
    all = all && s == VCLGB_SUCCESS;
    if (h_status) h_status[k] = s;
  }
  return all;
}

void batch_config(const Batch &bt, int *block, int *lanes) {
  if (block) *block = bt.block;
  if (lanes) *lanes = bt.lanes;
}

void batch_destroy(Batch *bt) { delete bt; }

}  // namespace vclgb
