// vecpass.cuh -- one generic grid-stride vector kernel with an optional fused
// deterministic reduction, and the iteration runner used by every solver.
#pragma once

#include "spmv.cuh"

namespace vclgb {

constexpr int kVecThreads = 256;

// F: NDOT, skip(), apply(i, dots), finalize(sums)
template <typename T, class F>
__global__ void __launch_bounds__(kVecThreads)
    vec_pass_kernel(size_t n, F f, T *partials, unsigned *counter) {
  pdl_trigger();
  pdl_wait();
  if (f.skip()) return;
  __shared__ T smem[DotArr<F::NDOT>::n * kVecThreads];
  T dots[DotArr<F::NDOT>::n];
#pragma unroll
  for (int i = 0; i < DotArr<F::NDOT>::n; ++i) dots[i] = T(0);
  const auto sc = f.load();  // per-thread copy of the step's device scalars
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  // two independent elements per step for memory-level parallelism
  for (; i + stride < n; i += 2 * stride) {
    f.apply(i, sc, dots);
    f.apply(i + stride, sc, dots);
  }
  if (i < n) f.apply(i, sc, dots);
  if constexpr (F::NDOT > 0) {
    T sums[F::NDOT];
    if (grid_reduce<F::NDOT, true>(dots, partials, counter, smem, sums)) f.finalize(sums);
  }
}

inline int vec_grid(const Backend &be, size_t n) { return waves_grid(be, kVecThreads, 8, n, 4); }

template <typename T, class F>
void vec_pass(Backend &be, size_t n, const F &f, const Reduction &red) {
  const int tp = timing_begin(be, 1);
  launch_kernel(be, vec_pass_kernel<T, F>,
                one_wave<vec_pass_kernel<T, F>>(be, vec_grid(be, n), kVecThreads), kVecThreads, 0,
                n, f, static_cast<T *>(red.partials), red.counter);
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  timing_end(be, tp);
}

// a single-thread device step (scalar bookkeeping between passes)
template <class F>
__global__ void scalar_step_kernel(F f) {
  if (threadIdx.x == 0 && blockIdx.x == 0) f();
}
template <class F>
void scalar_step(Backend &be, const F &f) {
  scalar_step_kernel<F><<<1, 32, 0, be.stream>>>(f);
  be.launches++;
  VCLGB_CHECK_LAUNCH();
}

// solver status words (device)
enum : int { kRunning = 0, kConverged = 1, kMaxIters = 2, kBreakdown = 3 };

// The condition of the solvers' device-side loop: another trip while the
// solve runs and fewer than `limit` trips were made (the count bounds the
// loop whatever the status word says).
static __global__ void loop_condition_kernel(cudaGraphConditionalHandle h, const int *done,
                                      unsigned *trips, unsigned limit) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const unsigned t = *trips + 1;
    *trips = t;
    cudaGraphSetConditional(h, (*done == kRunning && t < limit) ? 1u : 0u);
  }
}

// Launches `one_iteration` (which enqueues the kernels of one solver
// iteration and returns how many it launched) in chunks of check_every
// iterations, captured once into a CUDA graph and replayed; after every
// chunk the host reads the device status word.  Kernels of a finished solve
// return at their first instruction, so overshooting is harmless.
//
// Without kernel timing the chunk is the body of a device-side WHILE node
// (CUDA graph conditional node): the graph is launched once, the GPU repeats
// the chunk until the status word leaves kRunning (or the trip bound is
// reached), and the host waits once -- no status copy and no host round trip
// per chunk.  Launches with programmatic dependent launch (the optional PDL
// mode) keep the host-polled chunks.
template <class F>
void run_iterations(Backend &be, const int *d_done, uint32_t max_chunks_hint, uint32_t check_every,
                    bool use_graph, F &&one_iteration) {
  if (check_every == 0) check_every = 16;
  if (use_graph && !be.timing && !be.pdl) {
    const unsigned limit = max_chunks_hint + 4;
    if (!be.loop_trips.ptr) be.loop_trips.alloc(256, be.stream);
    unsigned *trips = be.loop_trips.as<unsigned>();
    cudaGraph_t graph = nullptr;
    VCLGB_CUDA(cudaGraphCreate(&graph, 0));
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&]() {
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
    };
    try {
      cudaGraphConditionalHandle handle;
      VCLGB_CUDA(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t node;
      VCLGB_CUDA(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      VCLGB_CUDA(cudaStreamBeginCaptureToGraph(be.stream, body, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
      const uint64_t before = be.launches;
      try {
        for (uint32_t i = 0; i < check_every; ++i) one_iteration();
        loop_condition_kernel<<<1, 32, 0, be.stream>>>(handle, d_done, trips, limit);
        VCLGB_CHECK_LAUNCH();
      } catch (...) {
        cudaGraph_t g2 = nullptr;
        cudaStreamEndCapture(be.stream, &g2);
        throw;
      }
      const uint64_t per_trip = be.launches - before + 1;
      be.launches = before;
      VCLGB_CUDA(cudaStreamEndCapture(be.stream, &body));
      VCLGB_CUDA(cudaGraphInstantiate(&exec, graph, 0));
      VCLGB_CUDA(cudaMemsetAsync(trips, 0, sizeof(unsigned), be.stream));
      VCLGB_CUDA(cudaGraphLaunch(exec, be.stream));
      VCLGB_CUDA(cudaMemcpyAsync(be.host_flags, d_done, sizeof(int), cudaMemcpyDeviceToHost,
                                 be.stream));
      VCLGB_CUDA(cudaMemcpyAsync(be.host_flags + 2, trips, sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, be.stream));
      VCLGB_CUDA(cudaStreamSynchronize(be.stream));
      be.launches += per_trip * (uint64_t)be.host_flags[2];
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
    if (be.host_flags[0] == kRunning)
      throw Error(VCLGB_TIMEOUT, "solver did not report completion within its iteration bound");
    be.tev_used = 0;
    return;
  }
  cudaGraphExec_t exec = nullptr;
  uint64_t per_chunk = 0;
  timing_collect(be, false);  // launches before the loop (timing on only)
  if (use_graph) {
    cudaGraph_t graph = nullptr;
    VCLGB_CUDA(cudaStreamBeginCapture(be.stream, cudaStreamCaptureModeThreadLocal));
    uint64_t before = be.launches;
    try {
      for (uint32_t i = 0; i < check_every; ++i) one_iteration();
    } catch (...) {
      cudaStreamEndCapture(be.stream, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    per_chunk = be.launches - before;
    be.launches = before;
    VCLGB_CUDA(cudaStreamEndCapture(be.stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    VCLGB_CUDA(e);
  }
  uint64_t chunks = 0;
  const uint64_t limit = (uint64_t)max_chunks_hint + 4;
  // One chunk is kept in flight ahead of the status check: chunk k+1 is
  // enqueued before the host waits for chunk k's status word, so the GPU
  // never idles while the host polls.  The chunk enqueued after convergence
  // costs only launches (its kernels return at their first instruction).
  // With kernel timing on, chunks run one at a time (timing_collect waits
  // for the stream and reads each replay's event pairs).
  const bool ahead = !be.timing;
  if (ahead && !be.poll_ev[0]) {
    for (int k = 0; k < 2; ++k)
      VCLGB_CUDA(cudaEventCreateWithFlags(&be.poll_ev[k], cudaEventDisableTiming));
  }
  auto enqueue = [&](uint64_t k) {
    if (exec) {
      VCLGB_CUDA(cudaGraphLaunch(exec, be.stream));
      be.launches += per_chunk;
    } else {
      for (uint32_t i = 0; i < check_every; ++i) one_iteration();
    }
    VCLGB_CUDA(cudaMemcpyAsync(be.host_flags + (k & 1), d_done, sizeof(int),
                               cudaMemcpyDeviceToHost, be.stream));
    if (ahead) VCLGB_CUDA(cudaEventRecord(be.poll_ev[k & 1], be.stream));
  };
  auto fail = [&]() {
    if (exec) cudaGraphExecDestroy(exec);
    throw Error(VCLGB_TIMEOUT, "solver did not report completion within its iteration bound");
  };
  if (ahead) {
    enqueue(0);
    for (uint64_t k = 0;; ++k) {
      enqueue(k + 1);
      VCLGB_CUDA(cudaEventSynchronize(be.poll_ev[k & 1]));
      ++chunks;
      if (be.host_flags[k & 1] != kRunning) break;
      if (chunks > limit) fail();
    }
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  } else {
    for (uint64_t k = 0;; ++k) {
      enqueue(k);
      VCLGB_CUDA(cudaStreamSynchronize(be.stream));
      timing_collect(be, exec != nullptr);  // graph events are replayed again
      ++chunks;
      if (be.host_flags[k & 1] != kRunning) break;
      if (chunks > limit) fail();
    }
  }
  if (exec) VCLGB_CUDA(cudaGraphExecDestroy(exec));
  be.tev_used = 0;
}

}  // namespace vclgb
