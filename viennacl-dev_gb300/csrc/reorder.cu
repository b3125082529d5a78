// reorder.cu -- bandwidth reduction (misc/cuthill_mckee.hpp) as a pre-pass for
// SpMV locality and shorter ILU0 level sets, and its application P A P^T on
// the GPU.
//
// The Cuthill-McKee orderings are sequential breadth-first searches: they run
// on the host over the CSR pattern (rows taken in ascending column order, the
// std::map order of the reference's host matrices) and follow
// reorder(matrix, cuthill_mckee_tag) (cuthill_mckee.hpp:366-421) and
// reorder(matrix, advanced_cuthill_mckee_tag) (cuthill_mckee.hpp:472-605)
// step for step -- root choice, queue order, the degree sort of each node's
// unnumbered neighbours (std::sort with the same comparison, so ties resolve
// as in the reference), and the advanced variant's search over root
// combinations scored by the resulting bandwidth -- so the permutations are
// identical.  The result maps node i to its new label perm[i].
//
// Applying a permutation, B = P A P^T with B(perm[i], perm[j]) = A(i, j), and
// measuring a bandwidth are data-parallel and run on the device.
#include <algorithm>
#include <deque>
#include <utility>
#include <vector>

#include "formats.hpp"

namespace vclgb {
namespace {

// the pattern with each row's columns ascending (duplicates merged)
struct Pattern {
  uint32_t n = 0;
  std::vector<uint32_t> rp, ci;
  uint32_t deg(uint32_t i) const { return rp[i + 1] - rp[i]; }
};

Pattern host_pattern(Backend &be, const Matrix &A) {
  Pattern g;
  g.n = A.rows;
  std::vector<uint32_t> rp(A.rows + 1), ci(A.nnz);
  VCLGB_CUDA(cudaMemcpyAsync(rp.data(), A.row_ptr, rp.size() * 4, cudaMemcpyDeviceToHost, be.stream));
  if (A.nnz)
    VCLGB_CUDA(cudaMemcpyAsync(ci.data(), A.col_idx, ci.size() * 4, cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  g.rp.assign(1, 0);
  g.ci.reserve(ci.size());
  for (uint32_t r = 0; r < A.rows; ++r) {
    const size_t b = g.ci.size();
    g.ci.insert(g.ci.end(), ci.begin() + rp[r], ci.begin() + rp[r + 1]);
    std::sort(g.ci.begin() + b, g.ci.end());
    g.ci.erase(std::unique(g.ci.begin() + b, g.ci.end()), g.ci.end());
    g.rp.push_back((uint32_t)g.ci.size());
  }
  return g;
}

// Breadth-first numbering from the queued roots: a node is numbered when it
// is first taken from the queue; its unnumbered neighbours are queued by
// increasing degree (cuthill_mckee.hpp:286-340).  Returns the next label.
uint32_t cm_component(const Pattern &g, std::deque<uint32_t> &queue, std::vector<bool> &done,
                      std::vector<uint32_t> &perm, uint32_t next,
                      std::vector<std::pair<uint32_t, uint32_t>> &scratch) {
  while (!queue.empty()) {
    const uint32_t node = queue.front();
    queue.pop_front();
    if (done[node]) continue;
    perm[node] = next++;
    done[node] = true;
    size_t m = 0;
    for (uint32_t k = g.rp[node]; k < g.rp[node + 1]; ++k) {
      const uint32_t nb = g.ci[k];
      if (!done[nb]) scratch[m++] = {nb, g.deg(nb)};
    }
    std::sort(scratch.begin(), scratch.begin() + (std::ptrdiff_t)m,
              [](const std::pair<uint32_t, uint32_t> &a, const std::pair<uint32_t, uint32_t> &b) {
                return a.second < b.second;
              });
    for (size_t i = 0; i < m; ++i) queue.push_back(scratch[i].first);
  }
  return next;
}

std::vector<uint32_t> cuthill_mckee(const Pattern &g) {
  const uint32_t n = g.n;
  std::vector<uint32_t> perm(n, 0);
  std::vector<bool> done(n, false);
  std::vector<std::pair<uint32_t, uint32_t>> scratch(n);
  std::deque<uint32_t> queue;
  uint32_t next = 0;
  while (next < n) {
    // isolated nodes (the diagonal alone) are numbered on sight; the root of
    // the next component is the first unnumbered node of least degree
    bool found = false;
    uint32_t root = 0, root_deg = n;
    for (uint32_t i = 0; i < n; ++i) {
      if (done[i]) continue;
      if (g.deg(i) == 1) {
        perm[i] = next++;
        done[i] = true;
        continue;
      }
      if (!found || g.deg(i) < root_deg) {
        root = i;
        root_deg = g.deg(i);
        found = true;
      }
    }
    if (!found) break;
    queue.push_back(root);
    next = cm_component(g, queue, done, perm, next, scratch);
  }
  return perm;
}

// the nodes reachable from `list` (breadth-first, cuthill_mckee.hpp:214-258)
void component_nodes(const Pattern &g, std::vector<uint32_t> &list) {
  std::vector<bool> seen(g.n, false);
  std::deque<uint32_t> queue(list.begin(), list.end());
  list.clear();
  while (!queue.empty()) {
    const uint32_t node = queue.front();
    queue.pop_front();
    if (seen[node]) continue;
    list.push_back(node);
    seen[node] = true;
    for (uint32_t k = g.rp[node]; k < g.rp[node + 1]; ++k) {
      const uint32_t nb = g.ci[k];
      if (nb != node && !seen[nb]) queue.push_back(nb);
    }
  }
}

// bandwidth among the numbered nodes (cuthill_mckee.hpp:46-76)
uint32_t numbered_bandwidth(const Pattern &g, const std::vector<bool> &done,
                            const std::vector<uint32_t> &perm) {
  uint32_t bw = 0;
  for (uint32_t i = 0; i < g.n; ++i) {
    if (!done[i]) continue;
    uint32_t lo = g.n, hi = 0;
    for (uint32_t k = g.rp[i]; k < g.rp[i + 1]; ++k) {
      const uint32_t c = g.ci[k];
      if (!done[c]) continue;
      hi = std::max(hi, perm[c]);
      lo = std::min(lo, perm[c]);
    }
    if (hi > lo) bw = std::max(bw, hi - lo);
  }
  return bw;
}

// next combination of comb.size() indices out of n in lexicographic order
// (cuthill_mckee.hpp:88-113)
bool next_combination(std::vector<uint32_t> &comb, size_t n) {
  const size_t m = comb.size();
  size_t k = m;
  while (k > 0 && ((k == m && comb[k - 1] == (uint32_t)n - 1) ||
                   (k < m && comb[k - 1] == comb[k] - 1)))
    --k;
  if (k == 0) return false;
  comb[k - 1] += 1;
  for (size_t i = k; i < m; ++i) comb[i] = comb[k - 1] + (uint32_t)(i - k);
  return true;
}

// every combination of up to gmax roots among the nodes of degree at most
// deg_min + a (deg_max - deg_min) of each component; the numbering with the
// smallest bandwidth is kept
std::vector<uint32_t> advanced_cuthill_mckee(const Pattern &g, double a, uint64_t gmax) {
  const uint32_t n = g.n;
  std::vector<uint32_t> perm(n, 0);
  std::vector<bool> done(n, false);
  std::vector<uint32_t> comp, roots, comb;
  std::vector<std::pair<uint32_t, uint32_t>> scratch(n);
  uint32_t next = 0;
  while (next < n) {
    comp.clear();
    for (uint32_t i = 0; i < n; ++i)
      if (!done[i]) {
        comp.push_back(i);
        component_nodes(g, comp);
        break;
      }
    uint64_t dmin = 0, dmax = 0;
    for (uint32_t v : comp) {
      const uint64_t d = g.deg(v);
      if (dmin == 0 || d < dmin) dmin = d;
      if (dmax == 0 || d > dmax) dmax = d;
    }
    const uint64_t da = dmin + (uint64_t)(a * double(dmax - dmin));
    roots.clear();
    for (uint32_t v : comp)
      if (g.deg(v) <= da) roots.push_back(v);
    const std::vector<bool> done0 = done;
    const std::vector<uint32_t> perm0 = perm;
    const uint32_t next0 = next;
    std::vector<bool> done_best;
    std::vector<uint32_t> perm_best = perm;
    uint32_t bw_best = 0;
    size_t gsz = 1;
    comb.assign(1, 0);
    for (;;) {
      done = done0;
      perm = perm0;
      std::deque<uint32_t> queue;
      for (uint32_t c : comb) queue.push_back(roots[c]);
      next = cm_component(g, queue, done, perm, next0, scratch);
      const uint32_t bw = numbered_bandwidth(g, done, perm);
      if (bw_best == 0 || bw < bw_best) {
        perm_best = perm;
        bw_best = bw;
        done_best = done;
      }
      if (!next_combination(comb, roots.size())) {
        ++gsz;
        if ((gmax > 0 && gsz > gmax) || gsz > roots.size()) break;
        comb.resize(gsz);
        for (size_t i = 0; i < gsz; ++i) comb[i] = (uint32_t)i;
      }
    }
    perm = perm_best;
    done = done_best;
  }
  return perm;
}

// ---- device side ------------------------------------------------------------
__global__ void permuted_lengths_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                        const uint32_t *__restrict__ perm, uint32_t *len) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows;
       i += (size_t)gridDim.x * blockDim.x)
    len[perm[i]] = rp[i + 1] - rp[i];
}

// Entry k of old row i goes to new row perm[i] at the rank of its new column
// among the row's entries (ties by position): columns ascending in every row.
template <typename V>
__global__ void permute_entries_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                       const uint32_t *__restrict__ ci, const V *__restrict__ v,
                                       const uint32_t *__restrict__ perm,
                                       const uint32_t *__restrict__ nrp, uint32_t *nci, V *nv) {
  const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t lane = threadIdx.x & 31;
  for (size_t i = warp; i < rows; i += nwarps) {  // one warp per old row
    const uint32_t b = rp[i], e = rp[i + 1], out = nrp[perm[i]];
    for (uint32_t k = b + lane; k < e; k += 32) {
      const uint32_t c = perm[ci[k]];
      uint32_t rank = 0;
      for (uint32_t q = b; q < e; ++q) {
        const uint32_t cq = perm[ci[q]];
        rank += (cq < c) || (cq == c && q < k);
      }
      nci[out + rank] = c;
      nv[out + rank] = v[k];
    }
  }
}

__global__ void bandwidth_kernel(uint32_t rows, const uint32_t *__restrict__ rp,
                                 const uint32_t *__restrict__ ci, unsigned *bw) {
  unsigned best = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows;
       i += (size_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0xffffffffu, hi = 0;
    for (uint32_t k = rp[i]; k < rp[i + 1]; ++k) {
      lo = min(lo, ci[k]);
      hi = max(hi, ci[k]);
    }
    if (hi > lo) best = max(best, hi - lo);
  }
  for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best) atomicMax(bw, best);
}

}  // namespace

void cuthill_mckee_perm(Backend &be, const Matrix &A, bool advanced, double a, uint64_t gmax,
                        uint32_t *d_perm) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "reordering takes a compressed_matrix");
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "reordering needs a square matrix");
  require(d_perm != nullptr || A.rows == 0, VCLGB_INVALID_ARGUMENT, "perm is NULL");
  if (A.rows == 0) return;
  const Pattern g = host_pattern(be, A);
  const std::vector<uint32_t> perm = advanced ? advanced_cuthill_mckee(g, a, gmax) : cuthill_mckee(g);
  VCLGB_CUDA(cudaMemcpyAsync(d_perm, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
}

std::unique_ptr<Matrix> csr_permute(Backend &be, const Matrix &A, const uint32_t *d_perm) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "permute takes a compressed_matrix");
  require(A.rows == A.cols, VCLGB_INVALID_ARGUMENT, "P A P^T needs a square matrix");
  require(d_perm != nullptr || A.rows == 0, VCLGB_INVALID_ARGUMENT, "perm is NULL");
  auto m = std::make_unique<Matrix>();
  m->format = VCLGB_CSR;
  m->prec = A.prec;
  m->rows = m->cols = A.rows;
  m->nnz = A.nnz;
  const uint32_t n = A.rows;
  m->own_row_ptr.alloc(((size_t)n + 1) * 4, be.stream);
  m->own_col_idx.alloc(std::max<uint64_t>(A.nnz, 1) * 4, be.stream);
  m->own_values.alloc(std::max<uint64_t>(A.nnz, 1) * A.vsize(), be.stream);
  if (n) {
    // perm must be a permutation: each new row receives exactly one old row
    DevBuf len(((size_t)n) * 4, be.stream), seen(((size_t)n) * 4, be.stream);
    VCLGB_CUDA(cudaMemsetAsync(len.ptr, 0, len.bytes, be.stream));
    std::vector<uint32_t> hp(n);
    VCLGB_CUDA(cudaMemcpyAsync(hp.data(), d_perm, (size_t)n * 4, cudaMemcpyDeviceToHost, be.stream));
    VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    std::vector<char> hit(n, 0);
    for (uint32_t i = 0; i < n; ++i) {
      require(hp[i] < n && !hit[hp[i]], VCLGB_INVALID_ARGUMENT, "perm is not a permutation");
      hit[hp[i]] = 1;
    }
    int g = waves_grid(be, 256, 8, n);
    permuted_lengths_kernel<<<g, 256, 0, be.stream>>>(n, A.row_ptr, d_perm, len.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
    extern_scan_u32(be, len.as<uint32_t>(), n, m->own_row_ptr.as<uint32_t>());
    int gw = waves_grid(be, 256, 8, (size_t)n * 32);
    if (A.prec == VCLGB_FLOAT64)
      permute_entries_kernel<uint64_t><<<gw, 256, 0, be.stream>>>(
          n, A.row_ptr, A.col_idx, static_cast<const uint64_t *>(A.values), d_perm,
          m->own_row_ptr.as<uint32_t>(), m->own_col_idx.as<uint32_t>(),
          m->own_values.as<uint64_t>());
    else
      permute_entries_kernel<uint32_t><<<gw, 256, 0, be.stream>>>(
          n, A.row_ptr, A.col_idx, static_cast<const uint32_t *>(A.values), d_perm,
          m->own_row_ptr.as<uint32_t>(), m->own_col_idx.as<uint32_t>(),
          m->own_values.as<uint32_t>());
    be.launches++;
    VCLGB_CHECK_LAUNCH();
  } else {
    VCLGB_CUDA(cudaMemsetAsync(m->own_row_ptr.ptr, 0, 4, be.stream));
  }
  m->row_ptr = m->own_row_ptr.as<uint32_t>();
  m->col_idx = m->own_col_idx.as<uint32_t>();
  m->values = m->own_values.ptr;
  csr_analyse(be, *m);
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  return m;
}

uint32_t csr_bandwidth(Backend &be, const Matrix &A) {
  require(A.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "bandwidth takes a compressed_matrix");
  if (A.rows == 0) return 0;
  DevBuf bw(sizeof(unsigned), be.stream);
  VCLGB_CUDA(cudaMemsetAsync(bw.ptr, 0, sizeof(unsigned), be.stream));
  int g = waves_grid(be, 256, 8, A.rows);
  bandwidth_kernel<<<g, 256, 0, be.stream>>>(A.rows, A.row_ptr, A.col_idx, bw.as<unsigned>());
  be.launches++;
  VCLGB_CHECK_LAUNCH();
  unsigned h = 0;
  VCLGB_CUDA(cudaMemcpyAsync(&h, bw.ptr, sizeof(h), cudaMemcpyDeviceToHost, be.stream));
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  return h;
}

}  // namespace vclgb
