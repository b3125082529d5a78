// ref_driver.cpp -- runs ViennaCL's own host/OpenMP backend on inputs stored
// as raw little-endian arrays in a directory, and writes its outputs there.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile against the ViennaCL
// headers (REF=<viennacl source tree>) into oracle/_ref/; used to pin the C
// restatement in vcl_oracle.c and to generate the golden fixtures under
// tests/golden/.  Nothing in the GPU engine includes or links it.
//
// Input directory layout:
//   meta.txt : "n ncols nnz"
//   rp.u32 (n+1), ci.u32 (nnz), v.f64 (nnz), b.f64 (n, optional), y0.f64 (optional)
// Commands (argv[1]) and outputs are listed in main() below.

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "viennacl/compressed_matrix.hpp"
#include "viennacl/coordinate_matrix.hpp"
#include "viennacl/ell_matrix.hpp"
#include "viennacl/hyb_matrix.hpp"
#include "viennacl/linalg/bicgstab.hpp"
#include "viennacl/linalg/cg.hpp"
#include "viennacl/linalg/gmres.hpp"
#include "viennacl/linalg/ilu.hpp"
#include "viennacl/linalg/jacobi_precond.hpp"
#include "viennacl/linalg/mixed_precision_cg.hpp"
#include "viennacl/linalg/prod.hpp"
#include "viennacl/linalg/row_scaling.hpp"
#include "viennacl/io/matrix_market.hpp"
#include "viennacl/misc/cuthill_mckee.hpp"
#include "viennacl/sliced_ell_matrix.hpp"
#include "viennacl/tools/adapter.hpp"
#include "viennacl/vector.hpp"

namespace {

std::string g_dir;

template <typename T>
std::vector<T> load(const std::string &name, size_t count, bool optional = false) {
  std::vector<T> out(count);
  std::ifstream f(g_dir + "/" + name, std::ios::binary);
  if (!f) {
    if (optional) return std::vector<T>();
    std::fprintf(stderr, "missing %s\n", name.c_str());
    std::exit(2);
  }
  f.read(reinterpret_cast<char *>(out.data()), sizeof(T) * count);
  return out;
}

template <typename T>
void save(const std::string &name, const T *data, size_t count) {
  std::ofstream f(g_dir + "/" + name, std::ios::binary);
  f.write(reinterpret_cast<const char *>(data), sizeof(T) * count);
}

template <typename T>
const T *raw(viennacl::backend::mem_handle const &h) {
  return viennacl::linalg::host_based::detail::extract_raw_pointer<T>(h);
}

struct Csr {
  size_t n, ncols, nnz;
  std::vector<unsigned> rp, ci;
  std::vector<double> v;
};

Csr load_csr() {
  Csr A;
  std::ifstream m(g_dir + "/meta.txt");
  m >> A.n >> A.ncols >> A.nnz;
  A.rp = load<unsigned>("rp.u32", A.n + 1);
  A.ci = load<unsigned>("ci.u32", A.nnz);
  A.v = load<double>("v.f64", A.nnz);
  return A;
}

template <typename T>
std::vector<std::map<unsigned, T> > to_maps(Csr const &A) {
  std::vector<std::map<unsigned, T> > M(A.n);
  for (size_t r = 0; r < A.n; ++r)
    for (unsigned k = A.rp[r]; k < A.rp[r + 1]; ++k) M[r][A.ci[k]] = T(A.v[k]);
  return M;
}

template <typename T>
void fill_matrix(Csr const &A, viennacl::compressed_matrix<T> &M) {
  std::vector<T> vals(A.v.begin(), A.v.end());
  M.set(A.rp.data(), A.ci.data(), vals.data(), A.n, A.ncols, A.nnz);
}

void to_vcl(std::vector<double> const &h, viennacl::vector<double> &d) {
  viennacl::fast_copy(h.begin(), h.end(), d.begin());
}

std::vector<double> from_vcl(viennacl::vector<double> const &d) {
  std::vector<double> h(d.size());
  viennacl::fast_copy(d.begin(), d.end(), h.begin());
  return h;
}

void write_info(unsigned long iters, double error, double seconds) {
  std::ofstream f(g_dir + "/info.txt");
  f.precision(17);
  f << iters << " " << error << " " << seconds << "\n";
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename Level>
void dump_levels(std::string const &prefix, Level const &row_index, Level const &row_buffers,
                 Level const &col_buffers, Level const &elem_buffers,
                 std::list<viennacl::vcl_size_t> const &nums) {
  // flattened: level_ptr, row_index, global row_ptr, cols, vals
  std::vector<unsigned> level_ptr(1, 0), rows, rowptr(1, 0), cols;
  std::vector<double> vals;
  typename Level::const_iterator a = row_index.begin(), b = row_buffers.begin(),
                                 c = col_buffers.begin(), d = elem_buffers.begin();
  std::list<viennacl::vcl_size_t>::const_iterator e = nums.begin();
  for (; a != row_index.end(); ++a, ++b, ++c, ++d, ++e) {
    size_t nr = *e;
    unsigned const *ri = raw<unsigned>(*a);
    unsigned const *rb = raw<unsigned>(*b);
    unsigned const *cb = raw<unsigned>(*c);
    double const *eb = raw<double>(*d);
    unsigned base = rowptr.back();
    for (size_t i = 0; i < nr; ++i) {
      rows.push_back(ri[i]);
      rowptr.push_back(base + rb[i + 1]);
    }
    for (unsigned k = 0; k < rb[nr]; ++k) {
      cols.push_back(cb[k]);
      vals.push_back(eb[k]);
    }
    level_ptr.push_back(static_cast<unsigned>(rows.size()));
  }
  save(prefix + "_level_ptr.u32", level_ptr.data(), level_ptr.size());
  save(prefix + "_row_index.u32", rows.data(), rows.size());
  save(prefix + "_row_ptr.u32", rowptr.data(), rowptr.size());
  save(prefix + "_cols.u32", cols.data(), cols.size());
  save(prefix + "_vals.f64", vals.data(), vals.size());
}

void dump_csr(std::string const &prefix, viennacl::compressed_matrix<double> const &M, size_t n) {
  save(prefix + "_rp.u32", raw<unsigned>(M.handle1()), n + 1);
  save(prefix + "_ci.u32", raw<unsigned>(M.handle2()), M.nnz());
  save(prefix + "_v.f64", raw<double>(M.handle()), M.nnz());
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_driver <cmd> <dir> [args]\n");
    return 2;
  }
  std::string cmd = argv[1];
  g_dir = argv[2];
  if (cmd == "mm_read") {  // args: file index_base -> mm_ret.u32, mm_rp.u32, mm_ci.u32, mm_v.f64
    std::vector<std::map<unsigned, double> > S;
    long ret = viennacl::io::read_matrix_market_file(S, argv[3], std::atol(argv[4]));
    std::vector<unsigned> rp(1, 0), ci;
    std::vector<double> v;
    for (size_t r = 0; r < S.size(); ++r) {
      for (std::map<unsigned, double>::const_iterator it = S[r].begin(); it != S[r].end(); ++it) {
        ci.push_back(it->first);
        v.push_back(it->second);
      }
      rp.push_back(static_cast<unsigned>(ci.size()));
    }
    unsigned meta[2] = {static_cast<unsigned>(ret), static_cast<unsigned>(S.size())};
    save("mm_ret.u32", meta, 2);
    save("mm_rp.u32", rp.data(), rp.size());
    save("mm_ci.u32", ci.data(), ci.size());
    save("mm_v.f64", v.data(), v.size());
    return 0;
  }
  Csr A = load_csr();
  size_t n = A.n;

  if (cmd == "spmv") {  // args: alpha beta -> y.f64
    double alpha = std::atof(argv[3]), beta = std::atof(argv[4]);
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    std::vector<double> xh = load<double>("x.f64", A.ncols);
    viennacl::vector<double> x(A.ncols), y(n);
    to_vcl(xh, x);
    std::vector<double> y0 = load<double>("y0.f64", n, true);
    if (!y0.empty()) to_vcl(y0, y);
    viennacl::linalg::prod_impl(M, x, alpha, y, beta);
    std::vector<double> yh = from_vcl(y);
    save("y.f64", yh.data(), n);
    unsigned const *blocks = raw<unsigned>(M.handle3());
    save("row_blocks.u32", blocks, M.blocks1() + 1);
  } else if (cmd == "spmv_f32") {  // -> yf.f32
    viennacl::compressed_matrix<float> M;
    fill_matrix(A, M);
    std::vector<double> xd = load<double>("x.f64", A.ncols);
    std::vector<float> xh(xd.begin(), xd.end());
    viennacl::vector<float> x(A.ncols), y(n);
    viennacl::fast_copy(xh.begin(), xh.end(), x.begin());
    y = viennacl::linalg::prod(M, x);
    std::vector<float> yh(n);
    viennacl::fast_copy(y.begin(), y.end(), yh.begin());
    save("yf.f32", yh.data(), n);
  } else if (cmd == "formats") {  // args: C hyb_threshold -> ell_*, sell_*, hyb_*, y_ell, y_hyb
    unsigned C = static_cast<unsigned>(std::atoi(argv[3]));
    double thr = std::atof(argv[4]);
    std::vector<std::map<unsigned, double> > S = to_maps<double>(A);
    viennacl::tools::const_sparse_matrix_adapter<double, unsigned> ad(S, n, A.ncols);
    std::vector<double> xh = load<double>("x.f64", A.ncols);
    viennacl::vector<double> x(A.ncols), y(n);
    to_vcl(xh, x);

    viennacl::ell_matrix<double> E;
    viennacl::copy(ad, E);
    unsigned w = static_cast<unsigned>(E.internal_maxnnz());
    save("ell_width.u32", &w, 1);
    save("ell_coords.u32", raw<unsigned>(E.handle2()), E.internal_nnz());
    save("ell_elems.f64", raw<double>(E.handle()), E.internal_nnz());
    y = viennacl::linalg::prod(E, x);
    std::vector<double> yh = from_vcl(y);
    save("y_ell.f64", yh.data(), n);

    viennacl::sliced_ell_matrix<double> Sl(n, A.ncols, C);
    viennacl::copy(ad, Sl);
    size_t nslices = (n - 1) / C + 1;
    unsigned const *cpb = raw<unsigned>(Sl.handle1());
    unsigned const *bs = raw<unsigned>(Sl.handle3());
    size_t total = size_t(bs[nslices - 1]) + size_t(cpb[nslices - 1]) * C;
    save("sell_cpb.u32", cpb, nslices);
    save("sell_bs.u32", bs, nslices);
    save("sell_cols.u32", raw<unsigned>(Sl.handle2()), total);
    save("sell_elems.f64", raw<double>(Sl.handle()), total);
    // the host SELL SpMV reads past the slice arrays when n % C == 0
    if (n % C != 0) {
      y = viennacl::linalg::prod(Sl, x);
      yh = from_vcl(y);
      save("y_sell.f64", yh.data(), n);
    }

    viennacl::hyb_matrix<double> H;
    H.csr_threshold(thr);
    viennacl::copy(ad, H);
    unsigned hw = static_cast<unsigned>(H.internal_ellnnz());
    unsigned tn = static_cast<unsigned>(H.csr_nnz());
    save("hyb_width.u32", &hw, 1);
    save("hyb_tail_nnz.u32", &tn, 1);
    save("hyb_ell_coords.u32", raw<unsigned>(H.handle2()), size_t(n) * hw);
    save("hyb_ell_elems.f64", raw<double>(H.handle()), size_t(n) * hw);
    save("hyb_tail_rp.u32", raw<unsigned>(H.handle3()), n + 1);
    save("hyb_tail_ci.u32", raw<unsigned>(H.handle4()), tn);
    save("hyb_tail_v.f64", raw<double>(H.handle5()), tn);
    y = viennacl::linalg::prod(H, x);
    yh = from_vcl(y);
    save("y_hyb.f64", yh.data(), n);
  } else if (cmd == "coo") {  // args: alpha beta -> coo_coords, coo_elems, coo_groups, y_coo
    double alpha = std::atof(argv[3]), beta = std::atof(argv[4]);
    std::vector<std::map<unsigned, double> > S = to_maps<double>(A);
    viennacl::tools::const_sparse_matrix_adapter<double, unsigned> ad(S, n, A.ncols);
    viennacl::coordinate_matrix<double> Co;
    viennacl::copy(ad, Co);
    size_t inz = Co.internal_nnz();
    unsigned meta[2] = {static_cast<unsigned>(Co.nnz()), static_cast<unsigned>(inz)};
    save("coo_nnz.u32", meta, 2);
    save("coo_coords.u32", raw<unsigned>(Co.handle12()), 2 * inz);
    save("coo_elems.f64", raw<double>(Co.handle()), inz);
    save("coo_groups.u32", raw<unsigned>(Co.handle3()), 65);
    std::vector<double> xh = load<double>("x.f64", A.ncols);
    viennacl::vector<double> x(A.ncols), y(n);
    to_vcl(xh, x);
    std::vector<double> y0 = load<double>("y0.f64", n, true);
    if (!y0.empty()) to_vcl(y0, y);
    viennacl::linalg::prod_impl(Co, x, alpha, y, beta);
    std::vector<double> yh = from_vcl(y);
    save("y_coo.f64", yh.data(), n);
  } else if (cmd == "hyb_f32_width") {  // args: thr -> hybf_width.u32
    double thr = std::atof(argv[3]);
    std::vector<std::map<unsigned, float> > S = to_maps<float>(A);
    viennacl::tools::const_sparse_matrix_adapter<float, unsigned> ad(S, n, A.ncols);
    viennacl::hyb_matrix<float> H;
    H.csr_threshold(static_cast<float>(thr));
    viennacl::copy(ad, H);
    unsigned hw = static_cast<unsigned>(H.internal_ellnnz());
    save("hybf_width.u32", &hw, 1);
  } else if (cmd == "cg" || cmd == "bicgstab" || cmd == "gmres" || cmd == "mixed_cg") {
    // args: tol maxit precond(none|jacobi|ilu0) [kdim | inner_tol]
    double tol = std::atof(argv[3]);
    unsigned maxit = static_cast<unsigned>(std::atoi(argv[4]));
    std::string pc = argc > 5 ? argv[5] : "none";
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    std::vector<double> bh = load<double>("b.f64", n);
    viennacl::vector<double> b(n), x(n);
    to_vcl(bh, b);
    unsigned long iters = 0;
    double err = 0, t0 = 0, t1 = 0;
    if (cmd == "cg") {
      viennacl::linalg::cg_tag tag(tol, maxit);
      if (pc == "jacobi") {
        viennacl::linalg::jacobi_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::jacobi_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc == "ilu0") {
        viennacl::linalg::ilu0_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::ilu0_tag(true));
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc.compare(0, 3, "row") == 0) {  // row0 / row1 / row2
        viennacl::linalg::row_scaling<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::row_scaling_tag(static_cast<unsigned>(pc[3] - '0')));
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc == "cpilu") {
        viennacl::linalg::chow_patel_ilu_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::chow_patel_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc.compare(0, 4, "bilu") == 0) {
        viennacl::linalg::block_ilu_precond<viennacl::compressed_matrix<double>,
                                            viennacl::linalg::ilu0_tag>
            P(M, viennacl::linalg::ilu0_tag(), static_cast<std::size_t>(std::atol(pc.c_str() + 4)));
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc == "cpicc") {
        viennacl::linalg::chow_patel_icc_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::chow_patel_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else {
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag);
        t1 = now();
      }
      iters = tag.iters();
      err = tag.error();
    } else if (cmd == "bicgstab") {
      viennacl::linalg::bicgstab_tag tag(tol, maxit);
      if (pc == "jacobi") {
        viennacl::linalg::jacobi_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::jacobi_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc.compare(0, 3, "row") == 0) {
        viennacl::linalg::row_scaling<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::row_scaling_tag(static_cast<unsigned>(pc[3] - '0')));
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc == "cpilu") {
        viennacl::linalg::chow_patel_ilu_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::chow_patel_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc.compare(0, 4, "bilu") == 0) {
        viennacl::linalg::block_ilu_precond<viennacl::compressed_matrix<double>,
                                            viennacl::linalg::ilu0_tag>
            P(M, viennacl::linalg::ilu0_tag(), static_cast<std::size_t>(std::atol(pc.c_str() + 4)));
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc == "cpicc") {
        viennacl::linalg::chow_patel_icc_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::chow_patel_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else {
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag);
        t1 = now();
      }
      iters = tag.iters();
      err = tag.error();
    } else if (cmd == "gmres") {
      unsigned kdim = argc > 6 ? static_cast<unsigned>(std::atoi(argv[6])) : 30;
      viennacl::linalg::gmres_tag tag(tol, maxit, kdim);
      if (pc == "jacobi") {
        viennacl::linalg::jacobi_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::jacobi_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc == "ilu0") {
        viennacl::linalg::ilu0_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::ilu0_tag(true));
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc.compare(0, 3, "row") == 0) {
        viennacl::linalg::row_scaling<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::row_scaling_tag(static_cast<unsigned>(pc[3] - '0')));
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else if (pc == "cpilu") {
        viennacl::linalg::chow_patel_ilu_precond<viennacl::compressed_matrix<double> > P(
            M, viennacl::linalg::chow_patel_tag());
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag, P);
        t1 = now();
      } else {
        t0 = now();
        x = viennacl::linalg::solve(M, b, tag);
        t1 = now();
      }
      iters = tag.iters();
      err = tag.error();
    } else {
      float inner = argc > 6 ? static_cast<float>(std::atof(argv[6])) : 1e-2f;
      viennacl::linalg::mixed_precision_cg_tag tag(tol, maxit, inner);
      t0 = now();
      x = viennacl::linalg::solve(M, b, tag);
      t1 = now();
      iters = tag.iters();
      err = tag.error();
    }
    std::vector<double> xh = from_vcl(x);
    save("x.f64", xh.data(), n);
    write_info(iters, err, t1 - t0);
  } else if (cmd == "trisolve") {  // -> tri_<tag>_<0|1>.f64: inplace_solve of b with A / trans(A)
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    std::vector<double> bh = load<double>("b.f64", n);
    const char *names[4] = {"lower", "upper", "unit_lower", "unit_upper"};
    for (int t = 0; t < 2; ++t)
      for (int tg = 0; tg < 4; ++tg) {
        viennacl::vector<double> z(n);
        to_vcl(bh, z);
        if (t == 0) {
          if (tg == 0) viennacl::linalg::inplace_solve(M, z, viennacl::linalg::lower_tag());
          if (tg == 1) viennacl::linalg::inplace_solve(M, z, viennacl::linalg::upper_tag());
          if (tg == 2) viennacl::linalg::inplace_solve(M, z, viennacl::linalg::unit_lower_tag());
          if (tg == 3) viennacl::linalg::inplace_solve(M, z, viennacl::linalg::unit_upper_tag());
        } else {
          if (tg == 0) viennacl::linalg::inplace_solve(trans(M), z, viennacl::linalg::lower_tag());
          if (tg == 1) viennacl::linalg::inplace_solve(trans(M), z, viennacl::linalg::upper_tag());
          if (tg == 2)
            viennacl::linalg::inplace_solve(trans(M), z, viennacl::linalg::unit_lower_tag());
          if (tg == 3)
            viennacl::linalg::inplace_solve(trans(M), z, viennacl::linalg::unit_upper_tag());
        }
        std::vector<double> zh = from_vcl(z);
        save(std::string("tri_") + names[tg] + "_" + char('0' + t) + ".f64", zh.data(), n);
      }
  } else if (cmd == "ilu0") {  // -> lu.f64, udiag.f64, L_*/U_* level arrays, z.f64 (apply to b)
    viennacl::compressed_matrix<double> LU;
    fill_matrix(A, LU);
    viennacl::linalg::precondition(LU, viennacl::linalg::ilu0_tag(true));
    save("lu.f64", raw<double>(LU.handle()), A.nnz);
    viennacl::vector<double> diag(n);
    viennacl::linalg::host_based::detail::row_info(LU, diag,
                                                   viennacl::linalg::detail::SPARSE_ROW_DIAGONAL);
    std::vector<double> dh = from_vcl(diag);
    save("udiag.f64", dh.data(), n);
    std::list<viennacl::backend::mem_handle> ri, rb, cb, eb;
    std::list<viennacl::vcl_size_t> nums;
    viennacl::linalg::detail::level_scheduling_setup_L(LU, diag, ri, rb, cb, eb, nums);
    dump_levels("L", ri, rb, cb, eb, nums);
    ri.clear(); rb.clear(); cb.clear(); eb.clear(); nums.clear();
    viennacl::linalg::detail::level_scheduling_setup_U(LU, diag, ri, rb, cb, eb, nums);
    dump_levels("U", ri, rb, cb, eb, nums);
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    viennacl::linalg::ilu0_precond<viennacl::compressed_matrix<double> > P(
        M, viennacl::linalg::ilu0_tag(true));
    std::vector<double> bh = load<double>("b.f64", n);
    viennacl::vector<double> z(n);
    to_vcl(bh, z);
    P.apply(z);
    std::vector<double> zh = from_vcl(z);
    save("z.f64", zh.data(), n);
  } else if (cmd == "chow_patel") {  // args: sweeps jacobi_iters -> cpl_*/cpu_* (ILU), icl_*/iclt_* (ICC), z
    viennacl::linalg::chow_patel_tag tag(static_cast<std::size_t>(std::atol(argv[3])),
                                         static_cast<std::size_t>(std::atol(argv[4])));
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    std::vector<double> bh = load<double>("b.f64", n);
    {
      viennacl::compressed_matrix<double> L, U;
      viennacl::vector<double> dL(n), dU(n);
      viennacl::linalg::detail::precondition(M, L, dL, U, dU, tag);
      dump_csr("cpl", L, n);
      dump_csr("cpu", U, n);
      std::vector<double> h = from_vcl(dL);
      save("cpl_diag.f64", h.data(), n);
      h = from_vcl(dU);
      save("cpu_diag.f64", h.data(), n);
      viennacl::linalg::chow_patel_ilu_precond<viennacl::compressed_matrix<double> > P(M, tag);
      viennacl::vector<double> z(n);
      to_vcl(bh, z);
      P.apply(z);
      h = from_vcl(z);
      save("cp_ilu_z.f64", h.data(), n);
    }
    {
      viennacl::compressed_matrix<double> L, Lt;
      viennacl::vector<double> dL(n);
      viennacl::linalg::detail::precondition(M, L, dL, Lt, tag);
      dump_csr("icl", L, n);
      dump_csr("iclt", Lt, n);
      std::vector<double> h = from_vcl(dL);
      save("icl_diag.f64", h.data(), n);
      viennacl::linalg::chow_patel_icc_precond<viennacl::compressed_matrix<double> > P(M, tag);
      viennacl::vector<double> z(n);
      to_vcl(bh, z);
      P.apply(z);
      h = from_vcl(z);
      save("cp_icc_z.f64", h.data(), n);
    }
  } else if (cmd == "block_ilu") {  // args: num_blocks -> bilu_lu.f64 (blocks' LU side by side), bilu_z.f64
    std::size_t nb = static_cast<std::size_t>(std::atol(argv[3]));
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    std::vector<double> lu_all;
    for (std::size_t i = 0; i < nb; ++i) {
      std::size_t s0 = (i * n) / nb, s1 = ((i + 1) * n) / nb;
      std::size_t bnnz = A.rp[s1] - A.rp[s0];
      viennacl::compressed_matrix<double> blk(s1 - s0, s1 - s0, bnnz);
      viennacl::linalg::detail::extract_block_matrix(M, blk, s0, s1);
      viennacl::linalg::precondition(blk, viennacl::linalg::ilu0_tag());
      double const *e = raw<double>(blk.handle());
      lu_all.insert(lu_all.end(), e, e + raw<unsigned>(blk.handle1())[s1 - s0]);
    }
    save("bilu_lu.f64", lu_all.data(), lu_all.size());
    viennacl::linalg::block_ilu_precond<viennacl::compressed_matrix<double>, viennacl::linalg::ilu0_tag>
        P(M, viennacl::linalg::ilu0_tag(), nb);
    std::vector<double> bh = load<double>("b.f64", n);
    viennacl::vector<double> z(n);
    to_vcl(bh, z);
    P.apply(z);
    std::vector<double> zh = from_vcl(z);
    save("bilu_z.f64", zh.data(), n);
  } else if (cmd == "row_norms") {  // -> norm0.f64, norm1.f64, norm2.f64 (row_info)
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    viennacl::linalg::detail::row_info_types sel[3] = {
        viennacl::linalg::detail::SPARSE_ROW_NORM_INF, viennacl::linalg::detail::SPARSE_ROW_NORM_1,
        viennacl::linalg::detail::SPARSE_ROW_NORM_2};
    for (int p = 0; p < 3; ++p) {
      viennacl::vector<double> d(n);
      viennacl::linalg::detail::row_info(M, d, sel[p]);
      std::vector<double> dh = from_vcl(d);
      save("norm" + std::to_string(p) + ".f64", dh.data(), n);
    }
  } else if (cmd == "cm") {  // args: advanced a gmax -> perm.u32, bw.u32 (before, after)
    std::vector<std::map<unsigned, double> > S = to_maps<double>(A);
    int advanced = std::atoi(argv[3]);
    std::vector<unsigned> perm;
    if (advanced)
      perm = viennacl::reorder(S, viennacl::advanced_cuthill_mckee_tag(
                                      std::atof(argv[4]), static_cast<std::size_t>(std::atol(argv[5]))));
    else
      perm = viennacl::reorder(S, viennacl::cuthill_mckee_tag());
    std::vector<bool> all(n, true);
    std::vector<unsigned> ident(n);
    for (size_t i = 0; i < n; ++i) ident[i] = static_cast<unsigned>(i);
    unsigned bw[2] = {viennacl::detail::calc_reordered_bw(S, all, ident),
                      viennacl::detail::calc_reordered_bw(S, all, perm)};
    save("perm.u32", perm.data(), n);
    save("bw.u32", bw, 2);
  } else if (cmd == "jacobi_diag") {  // -> diag.f64
    viennacl::compressed_matrix<double> M;
    fill_matrix(A, M);
    viennacl::vector<double> diag(n);
    viennacl::linalg::detail::row_info(M, diag, viennacl::linalg::detail::SPARSE_ROW_DIAGONAL);
    std::vector<double> dh = from_vcl(diag);
    save("diag.f64", dh.data(), n);
  } else {
    std::fprintf(stderr, "unknown command %s\n", cmd.c_str());
    return 2;
  }
  return 0;
}
