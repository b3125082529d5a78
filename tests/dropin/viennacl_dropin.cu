// A ViennaCL program written against ViennaCL's own API only.  Compiled with
// the engine's shadow headers first on the include path
// (viennacl-dev_gb300/shadow) and linked with libvclgb.so, its sparse products,
// vector updates, reductions and solves run in the engine; nothing here names
// the engine.  Writes y = A b, the vector expression results, the triangular
// solve and the three solves to argv[1] as raw doubles, and iteration counts
// to stdout.
#include <cstdio>
#include <map>
#include <vector>

#include "viennacl/compressed_matrix.hpp"
#include "viennacl/linalg/bicgstab.hpp"
#include "viennacl/linalg/cg.hpp"
#include "viennacl/linalg/gmres.hpp"
#include "viennacl/linalg/inner_prod.hpp"
#include "viennacl/linalg/jacobi_precond.hpp"
#include "viennacl/linalg/norm_2.hpp"
#include "viennacl/linalg/prod.hpp"
#include "viennacl/linalg/sparse_matrix_operations.hpp"
#include "viennacl/vector.hpp"

int main(int argc, char **argv) {
  const unsigned N = 48, n = N * N;
  // 2D convection-diffusion on an N x N grid (upwind in x), nonsymmetric
  std::vector<std::map<unsigned int, double> > A(n);
  for (unsigned j = 0; j < N; ++j)
    for (unsigned i = 0; i < N; ++i) {
      const unsigned r = j * N + i;
      A[r][r] = 4.5;
      if (i > 0) A[r][r - 1] = -1.4;
      if (i + 1 < N) A[r][r + 1] = -0.6;
      if (j > 0) A[r][r - N] = -1.0;
      if (j + 1 < N) A[r][r + N] = -1.0;
    }
  std::vector<double> hb(n);
  for (unsigned r = 0; r < n; ++r) hb[r] = 1.0 + 0.5 * ((r * 7919u) % 1000) / 1000.0;

  viennacl::compressed_matrix<double> vA;
  viennacl::copy(A, vA);
  viennacl::vector<double> b(n), y(n), v(n);
  viennacl::copy(hb, b);

  y = viennacl::linalg::prod(vA, b);                       // prod_impl
  v = 2.0 * y - b / 4.0;                                    // avbv
  v += 0.5 * b;                                             // avbv_v / av
  double ip = viennacl::linalg::inner_prod(v, b);           // inner_prod_cpu
  double nr = viennacl::linalg::norm_2(v);                  // norm_2_cpu
  viennacl::vector<double> e = viennacl::linalg::element_prod(v, b);  // element_op
  viennacl::vector<double> t = b;
  viennacl::linalg::inplace_solve(vA, t, viennacl::linalg::lower_tag());  // triangular solve

  viennacl::linalg::jacobi_precond<viennacl::compressed_matrix<double> > P(
      vA, viennacl::linalg::jacobi_tag());
  viennacl::linalg::cg_tag cg(1e-10, 2000);
  viennacl::vector<double> x1 = viennacl::linalg::solve(vA, b, cg, P);
  viennacl::linalg::bicgstab_tag bt(1e-10, 2000);
  viennacl::vector<double> x2 = viennacl::linalg::solve(vA, b, bt);
  viennacl::linalg::gmres_tag gt(1e-10, 2000, 30);
  viennacl::vector<double> x3 = viennacl::linalg::solve(vA, b, gt, P);

  std::vector<double> out;
  for (viennacl::vector<double> const *w : {&y, &v, &e, &t, &x1, &x2, &x3}) {
    std::vector<double> h(n);
    viennacl::copy(*w, h);
    out.insert(out.end(), h.begin(), h.end());
  }
  out.push_back(ip);
  out.push_back(nr);
  FILE *f = std::fopen(argc > 1 ? argv[1] : "dropin.f64", "wb");
  if (!f) return 2;
  std::fwrite(out.data(), sizeof(double), out.size(), f);
  std::fclose(f);
  std::printf("cg %u %.17g\nbicgstab %u %.17g\ngmres %u %.17g\n", cg.iters(), cg.error(),
              bt.iters(), bt.error(), gt.iters(), gt.error());
  return 0;
}
