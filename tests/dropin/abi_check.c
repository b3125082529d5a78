/* A plain C program that uses the engine only through include/vclgb.h and the
 * CUDA runtime's C API, as a C, Go (cgo) or Fortran binding would: it builds
 * the 2D 5-point Laplacian of an N x N grid (N = argv[2], default 40) in host
 * CSR arrays, copies them to the device, wraps them as a compressed_matrix,
 * runs one SpMV (y = A b) and a Jacobi-preconditioned CG solve (tolerance
 * 1e-10), and writes y then x (raw doubles) to argv[1]; the iteration count,
 * the solver's error estimate and the status go to stdout.  Exit status 0 only
 * if every call returned VCLGB_SUCCESS. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime.h>

#include "vclgb.h"

#define CHECK(call)                                                              \
  do {                                                                           \
    vclgbStatus s_ = (call);                                                     \
    if (s_ != VCLGB_SUCCESS) {                                                   \
      fprintf(stderr, "%s failed: %d (%s)\n", #call, (int)s_,                  \
              be ? vclgbBackendLastError(be) : "");                              \
      return 1;                                                                  \
    }                                                                            \
  } while (0)

int main(int argc, char **argv) {
  const uint32_t N = argc > 2 ? (uint32_t)atoi(argv[2]) : 40u, n = N * N;
  uint32_t *rp = malloc(sizeof(uint32_t) * (n + 1)), *ci = malloc(sizeof(uint32_t) * 5 * n);
  double *v = malloc(sizeof(double) * 5 * n), *b = malloc(sizeof(double) * n);
  double *out = malloc(sizeof(double) * 2 * n);
  uint32_t k = 0;
  rp[0] = 0;
  for (uint32_t j = 0; j < N; ++j)
    for (uint32_t i = 0; i < N; ++i) {
      const uint32_t r = j * N + i;
      if (j > 0) { ci[k] = r - N; v[k++] = -1.0; }
      if (i > 0) { ci[k] = r - 1; v[k++] = -1.0; }
      ci[k] = r; v[k++] = 4.0;
      if (i + 1 < N) { ci[k] = r + 1; v[k++] = -1.0; }
      if (j + 1 < N) { ci[k] = r + N; v[k++] = -1.0; }
      rp[r + 1] = k;
      b[r] = 1.0 + (double)((r * 7919u) % 1000u) / 1000.0;
    }
  vclgbBackend be = NULL;
  uint32_t *d_rp, *d_ci;
  double *d_v, *d_b, *d_y, *d_x;
  if (cudaMalloc((void **)&d_rp, 4 * (n + 1)) || cudaMalloc((void **)&d_ci, 4 * (size_t)k) ||
      cudaMalloc((void **)&d_v, 8 * (size_t)k) || cudaMalloc((void **)&d_b, 8 * (size_t)n) ||
      cudaMalloc((void **)&d_y, 8 * (size_t)n) || cudaMalloc((void **)&d_x, 8 * (size_t)n)) {
    fprintf(stderr, "cudaMalloc failed\n");
    return 1;
  }
  cudaMemcpy(d_rp, rp, 4 * (n + 1), cudaMemcpyHostToDevice);
  cudaMemcpy(d_ci, ci, 4 * (size_t)k, cudaMemcpyHostToDevice);
  cudaMemcpy(d_v, v, 8 * (size_t)k, cudaMemcpyHostToDevice);
  cudaMemcpy(d_b, b, 8 * (size_t)n, cudaMemcpyHostToDevice);

  vclgbMatrix A = NULL;
  vclgbPrecond P = NULL;
  vclgbSolverTag tag;
  CHECK(vclgbBackendCreate(&be, NULL));
  CHECK(vclgbCsrCreate(be, VCLGB_FLOAT64, n, n, k, d_rp, d_ci, d_v, &A));
  CHECK(vclgbSpmv(be, A, 1.0, d_b, 0, 1, 0.0, d_y, 0, 1));
  CHECK(vclgbJacobiCreate(be, A, &P));
  vclgbSolverTagInit(&tag, 0);
  tag.tol = 1e-10;
  tag.max_iters = 5000;
  CHECK(vclgbSolveCG(be, A, d_b, d_x, &tag, P));
  CHECK(vclgbBackendSynchronize(be));
  cudaMemcpy(out, d_y, 8 * (size_t)n, cudaMemcpyDeviceToHost);
  cudaMemcpy(out + n, d_x, 8 * (size_t)n, cudaMemcpyDeviceToHost);
  FILE *f = fopen(argc > 1 ? argv[1] : "abi_check.f64", "wb");
  if (!f) return 1;
  fwrite(out, sizeof(double), 2 * (size_t)n, f);
  fclose(f);
  printf("%s iters %u error %.17g status %u\n", vclgbVersion(), tag.iters, tag.error, tag.status);
  CHECK(vclgbPrecondDestroy(&P));
  CHECK(vclgbMatrixDestroy(&A));
  CHECK(vclgbBackendDestroy(&be));
  return tag.status == VCLGB_SUCCESS ? 0 : 1;
}
