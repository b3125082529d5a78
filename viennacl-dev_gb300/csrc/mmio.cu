// mmio.cu -- MatrixMarket reader and writer (io/matrix_market.hpp).
//
// The reader follows read_matrix_market_file_impl (io/matrix_market.hpp:101-326):
//   * lines are trimmed of leading/trailing spaces; empty lines are skipped
//     but counted; a line starting with '%' is a comment, "%%" a header;
//   * the header must read "MatrixMarket matrix coordinate <field> <symmetry>"
//     (case-insensitive) with field real | complex (real part kept) | pattern
//     (value 1) and symmetry general | symmetric; "array" and every other
//     word is rejected, as is a missing word (the reference then compares the
//     previous word again, which never matches);
//   * the first other line holds "rows cols nnz"; entries "row col [value]"
//     follow, index_base subtracted, out-of-range indices rejected;
//   * each entry assigns A(row, col) = value (and A(col, row) = value when
//     symmetric): a later assignment to the same position replaces the
//     earlier one, the std::map semantics of the reference's sparse matrix
//     adapter;
//   * reading stops after nnz entries; a file that ends before nnz entries is
//     an error (the reference fails its parse of the empty line at the end);
//     a size line with nnz = 0 gives an empty matrix (the reference reports a
//     failure there for the same reason);
//   * the return value is the number of lines read up to the last entry.
// Errors return VCLGB_INVALID_ARGUMENT with a message naming the file, the
// line and the cause in the backend's last error (the reference prints its
// message and returns 0).
//
// Differences kept on purpose: lines may be longer than the reference's
// 1024-character buffer; "%%" lines after the size line are comments; a
// malformed number is an error (the reference reads an uninitialised index).
//
// Text parsing is host work; the data region is split at line boundaries and
// parsed by all host threads, the entries are grouped by row with a stable
// counting sort, each row is ordered by column (later duplicates win), and
// the CSR arrays go to the device once, where the matrix is validated and
// analysed like any other compressed_matrix.
#include <algorithm>
#include <cctype>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "formats.hpp"

namespace vclgb {
namespace {

struct Entry {
  uint32_t row, col;
  double val;
};

Error mm_error(const std::string &msg) { return Error(VCLGB_INVALID_ARGUMENT, msg); }

std::string lower(std::string s) {
  for (char &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// [b, e) of the next line starting at p (without the '\n'); advances p
inline void next_line(const char *&p, const char *end, const char *&b, const char *&e) {
  b = p;
  const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
  e = nl ? nl : end;
  p = nl ? nl + 1 : end;
}

inline void trim(const char *&b, const char *&e) {
  while (b < e && *b == ' ') ++b;
  while (e > b && e[-1] == ' ') --e;
}

// whitespace-separated token starting at p; false when the line has no more
inline bool token(const char *&p, const char *e, const char *&tb, const char *&te) {
  while (p < e && std::isspace((unsigned char)*p)) ++p;
  if (p >= e) return false;
  tb = p;
  while (p < e && !std::isspace((unsigned char)*p)) ++p;
  te = p;
  return true;
}

template <typename V>
inline bool parse_num(const char *b, const char *e, V &out) {
  if (b < e && *b == '+') ++b;  // the reference's stream extraction accepts a leading '+'
  auto r = std::from_chars(b, e, out);
  return r.ec == std::errc() && r.ptr == e;
}

struct Header {
  bool symmetric = false, pattern = false;
  uint64_t rows = 0, cols = 0, nnz = 0;
};

// Parses the entry lines of [p, end): every entry, or stops at the first
// malformed line (err set, err_line = its index among this chunk's lines).
struct Chunk {
  std::vector<Entry> entries;
  uint64_t lines = 0;
  bool err = false;
  uint64_t err_line = 0;
  std::string msg;
};

template <typename V>
void parse_chunk(const char *p, const char *end, const Header &h, long index_base, Chunk &c) {
  const char *b, *e;
  while (p < end) {
    next_line(p, end, b, e);
    ++c.lines;
    trim(b, e);
    if (b == e || *b == '%') continue;
    const char *q = b, *tb, *te;
    long row = 0, col = 0;
    V val = V(1);
    if (!token(q, e, tb, te) || !parse_num(tb, te, row)) {
      c.msg = "Parse error for matrix row entry";
    } else if (!token(q, e, tb, te) || !parse_num(tb, te, col)) {
      c.msg = "Parse error for matrix col entry";
    } else if (!h.pattern && (!token(q, e, tb, te) || !parse_num(tb, te, val))) {
      c.msg = "Parse error for matrix entry";
    } else {
      row -= index_base;
      col -= index_base;
      if (row < 0 || (uint64_t)row >= h.rows) c.msg = "Row index out of bounds: " + std::to_string(row);
      else if (col < 0 || (uint64_t)col >= h.cols) c.msg = "Column index out of bounds: " + std::to_string(col);
    }
    if (!c.msg.empty()) {
      c.err = true;
      c.err_line = c.lines - 1;
      return;
    }
    c.entries.push_back({(uint32_t)row, (uint32_t)col, (double)val});
  }
}

struct Parsed {
  Header h;
  std::vector<Entry> entries;  // in file order
  uint64_t lines = 0;
};

template <typename V>
void parse_file(const char *path, long index_base, Parsed &out) {
  FILE *f = std::fopen(path, "rb");
  if (!f) throw mm_error(std::string("Matrix Market Reader: Cannot open file ") + path);
  std::vector<char> buf;
  {
    std::fseek(f, 0, SEEK_END);
    long sz = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(sz > 0 ? (size_t)sz : 0);
    size_t got = sz > 0 ? std::fread(buf.data(), 1, buf.size(), f) : 0;
    std::fclose(f);
    buf.resize(got);
  }
  const char *p = buf.data(), *end = buf.data() + buf.size();
  const std::string where = std::string("Error in file ") + path;
  Header &h = out.h;
  uint64_t line = 0;
  bool have_size = false;
  const char *b, *e;
  // header, comments and the size line
  while (p < end && !have_size) {
    next_line(p, end, b, e);
    ++line;
    trim(b, e);
    if (b == e) continue;
    if (*b == '%') {
      if (e - b < 2 || b[1] != '%') continue;
      const char *q = b + 2, *tb, *te;
      std::string tok;
      auto next = [&]() {
        if (token(q, e, tb, te)) tok.assign(tb, te);  // a missing word keeps the previous one
        return lower(tok);
      };
      const std::string at = where + " at line " + std::to_string(line) + ": ";
      if (next() != "matrixmarket") throw mm_error(at + "Expected 'MatrixMarket', got '" + tok + "'");
      if (next() != "matrix") throw mm_error(at + "Expected 'matrix', got '" + tok + "'");
      const std::string kind = next();
      if (kind == "array") throw mm_error(at + "'array' type is not supported yet!");
      if (kind != "coordinate")
        throw mm_error(at + "Expected 'array' or 'coordinate', got '" + tok + "'");
      const std::string field = next();
      if (field == "pattern") h.pattern = true;
      else if (field != "complex" && field != "real")
        throw mm_error(where + ": unsupported field '" + tok +
                       "' (real, complex or pattern matrices only)");
      const std::string sym = next();
      if (sym == "symmetric") h.symmetric = true;
      else if (sym != "general")
        throw mm_error(where + ": unsupported symmetry '" + tok +
                       "' (general or symmetric matrices only)");
      continue;
    }
    const char *q = b, *tb, *te;
    const std::string at = where + ": Could not get matrix dimensions ";
    if (!token(q, e, tb, te) || !parse_num(tb, te, h.rows))
      throw mm_error(at + "(rows) in line " + std::to_string(line));
    if (!token(q, e, tb, te) || !parse_num(tb, te, h.cols))
      throw mm_error(at + "(columns) in line " + std::to_string(line));
    if (!token(q, e, tb, te) || !parse_num(tb, te, h.nnz))
      throw mm_error(at + "(columns) in line " + std::to_string(line));
    have_size = true;
  }
  if (!have_size) throw mm_error(where + ": Could not get matrix dimensions (rows) in line " +
                                 std::to_string(line + 1));
  if (h.rows == 0 || h.cols == 0) h.rows = h.cols = 0;  // the reference resizes only for both > 0
  require(h.rows <= 0xffffffffull && h.cols <= 0xffffffffull, VCLGB_INVALID_ARGUMENT,
          "matrix dimensions exceed 32-bit indices");
  // data region: chunks split at line boundaries, parsed in parallel
  const size_t bytes = (size_t)(end - p);
  unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  if (bytes < (4u << 20)) nt = 1;
  std::vector<const char *> cut(nt + 1);
  cut[0] = p;
  cut[nt] = end;
  for (unsigned t = 1; t < nt; ++t) {
    const char *c = p + bytes * t / nt;
    if (c < cut[t - 1]) c = cut[t - 1];
    const char *nl = static_cast<const char *>(std::memchr(c, '\n', (size_t)(end - c)));
    cut[t] = nl ? nl + 1 : end;
  }
  std::vector<Chunk> chunks(nt);
  {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t)
      th.emplace_back([&, t]() { parse_chunk<V>(cut[t], cut[t + 1], h, index_base, chunks[t]); });
    parse_chunk<V>(cut[0], cut[1], h, index_base, chunks[0]);
    for (auto &x : th) x.join();
  }
  // entries in file order up to nnz; the first error before that is fatal
  out.lines = line;
  if (h.nnz == 0) return;  // (the reference reports a failure for an empty matrix)
  out.entries.reserve(std::min<uint64_t>(h.nnz, 1ull << 32));
  for (unsigned t = 0; t < nt; ++t) {
    const Chunk &c = chunks[t];
    const uint64_t need = h.nnz - out.entries.size();
    if (c.entries.size() >= need) {
      // the nnz-th entry lies in this chunk: count the lines up to it
      out.entries.insert(out.entries.end(), c.entries.begin(), c.entries.begin() + need);
      const char *q = cut[t];
      for (uint64_t seen = 0; seen < need;) {
        next_line(q, cut[t + 1], b, e);
        ++line;
        trim(b, e);
        if (b != e && *b != '%') ++seen;
      }
      out.lines = line;
      return;
    }
    out.entries.insert(out.entries.end(), c.entries.begin(), c.entries.end());
    if (c.err)
      throw mm_error(where + ": " + c.msg + " in line " + std::to_string(line + c.err_line + 1));
    line += c.lines;
  }
  throw mm_error(where + ": Parse error for matrix row entry in line " + std::to_string(line + 1) +
                 " (the file ends after " + std::to_string(out.entries.size()) + " of " +
                 std::to_string(h.nnz) + " entries)");
}

// CSR of the assignments in order: A(r, c) = v, A(c, r) = v when symmetric;
// the last assignment to a position wins; columns ascending in each row.
void assemble(const Parsed &in, std::vector<uint32_t> &rp, std::vector<uint32_t> &ci,
              std::vector<double> &v) {
  const uint64_t n = in.h.rows;
  const bool sym = in.h.symmetric;
  // writes in order: entry k gives write 2k (r, c) and, if symmetric, 2k+1 (c, r)
  std::vector<uint64_t> cnt(n + 1, 0);
  for (const Entry &x : in.entries) {
    ++cnt[x.row];
    if (sym) ++cnt[x.col];
  }
  std::vector<uint64_t> off(n + 1, 0);
  for (uint64_t r = 0; r < n; ++r) off[r + 1] = off[r] + cnt[r];
  struct W { uint32_t col; double val; };
  std::vector<W> w(off[n]);
  {
    std::vector<uint64_t> cur(off.begin(), off.end() - 1);
    for (const Entry &x : in.entries) {  // rows keep the write order (stable)
      w[cur[x.row]++] = {x.col, x.val};
      if (sym) w[cur[x.col]++] = {x.row, x.val};
    }
  }
  // per row: stable order by column (equal columns keep write order), then
  // keep the last write of each column
  std::vector<uint32_t> len(n, 0);
  unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  if (w.size() < (1u << 20)) nt = 1;
  auto work = [&](unsigned t) {
    for (uint64_t r = n * t / nt; r < n * (t + 1) / nt; ++r) {
      W *a = w.data() + off[r], *z = w.data() + off[r + 1];
      std::stable_sort(a, z, [](const W &x, const W &y) { return x.col < y.col; });
      uint64_t k = 0;
      for (W *it = a; it < z; ++it) {
        if (it + 1 < z && it[1].col == it->col) continue;  // a later write replaces it
        a[k++] = *it;
      }
      len[r] = (uint32_t)k;
    }
  };
  {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
  }
  uint64_t total = 0;
  for (uint64_t r = 0; r < n; ++r) total += len[r];
  require(total <= 0xffffffffull, VCLGB_INVALID_ARGUMENT, "more than 2^32 - 1 entries");
  rp.assign(n + 1, 0);
  for (uint64_t r = 0; r < n; ++r) rp[r + 1] = rp[r] + len[r];
  ci.resize(rp[n]);
  v.resize(rp[n]);
  for (uint64_t r = 0; r < n; ++r)
    for (uint32_t k = 0; k < len[r]; ++k) {
      ci[rp[r] + k] = w[off[r] + k].col;
      v[rp[r] + k] = w[off[r] + k].val;
    }
}

}  // namespace

std::unique_ptr<Matrix> read_matrix_market(Backend &be, const char *path, long index_base,
                                           vclgbPrecision prec, uint64_t *lines_read) {
  require(path != nullptr, VCLGB_INVALID_ARGUMENT, "path is NULL");
  Parsed in;
  if (prec == VCLGB_FLOAT32) parse_file<float>(path, index_base, in);
  else parse_file<double>(path, index_base, in);
  std::vector<uint32_t> rp, ci;
  std::vector<double> v;
  assemble(in, rp, ci, v);
  auto m = std::make_unique<Matrix>();
  m->format = VCLGB_CSR;
  m->prec = prec;
  m->rows = (uint32_t)in.h.rows;
  m->cols = (uint32_t)in.h.cols;
  m->nnz = ci.size();
  const size_t vs = m->vsize();
  m->own_row_ptr.alloc(rp.size() * 4, be.stream);
  m->own_col_idx.alloc(std::max<size_t>(ci.size(), 1) * 4, be.stream);
  m->own_values.alloc(std::max<size_t>(v.size(), 1) * vs, be.stream);
  VCLGB_CUDA(cudaMemcpyAsync(m->own_row_ptr.ptr, rp.data(), rp.size() * 4, cudaMemcpyHostToDevice,
                             be.stream));
  if (!ci.empty()) {
    VCLGB_CUDA(cudaMemcpyAsync(m->own_col_idx.ptr, ci.data(), ci.size() * 4,
                               cudaMemcpyHostToDevice, be.stream));
    if (prec == VCLGB_FLOAT32) {
      std::vector<float> vf(v.begin(), v.end());  // exact: the values were parsed as float
      VCLGB_CUDA(cudaMemcpyAsync(m->own_values.ptr, vf.data(), vf.size() * 4,
                                 cudaMemcpyHostToDevice, be.stream));
      VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    } else {
      VCLGB_CUDA(cudaMemcpyAsync(m->own_values.ptr, v.data(), v.size() * 8,
                                 cudaMemcpyHostToDevice, be.stream));
    }
  }
  m->row_ptr = m->own_row_ptr.as<uint32_t>();
  m->col_idx = m->own_col_idx.as<uint32_t>();
  m->values = m->own_values.ptr;
  csr_validate(be, *m);
  csr_analyse(be, *m);
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  if (lines_read) *lines_read = in.lines;
  return m;
}

// write_matrix_market_file_impl (io/matrix_market.hpp:374-399): the header
// "%%MatrixMarket matrix coordinate real general", "rows cols nnz", then one
// "row col value" line per stored entry in row order; values are printed with
// `digits` significant digits (6, the reference's stream default, when 0).
void write_matrix_market(Backend &be, const Matrix &m, const char *path, long index_base,
                         int digits) {
  require(path != nullptr, VCLGB_INVALID_ARGUMENT, "path is NULL");
  require(m.format == VCLGB_CSR, VCLGB_INVALID_ARGUMENT, "the writer takes a compressed_matrix");
  require(digits >= 0 && digits <= 17, VCLGB_INVALID_ARGUMENT, "digits must be 0..17");
  std::vector<uint32_t> rp(m.rows + 1), ci(m.nnz);
  std::vector<double> v(m.nnz);
  VCLGB_CUDA(cudaMemcpyAsync(rp.data(), m.row_ptr, rp.size() * 4, cudaMemcpyDeviceToHost, be.stream));
  if (m.nnz) {
    VCLGB_CUDA(cudaMemcpyAsync(ci.data(), m.col_idx, ci.size() * 4, cudaMemcpyDeviceToHost, be.stream));
    if (m.prec == VCLGB_FLOAT64) {
      VCLGB_CUDA(cudaMemcpyAsync(v.data(), m.values, v.size() * 8, cudaMemcpyDeviceToHost, be.stream));
      VCLGB_CUDA(cudaStreamSynchronize(be.stream));
    } else {
      std::vector<float> vf(m.nnz);
      VCLGB_CUDA(cudaMemcpyAsync(vf.data(), m.values, vf.size() * 4, cudaMemcpyDeviceToHost, be.stream));
      VCLGB_CUDA(cudaStreamSynchronize(be.stream));
      std::copy(vf.begin(), vf.end(), v.begin());
    }
  }
  VCLGB_CUDA(cudaStreamSynchronize(be.stream));
  FILE *f = std::fopen(path, "w");
  require(f != nullptr, VCLGB_INVALID_ARGUMENT, "cannot open the output file");
  const int prec = digits ? digits : 6;
  std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n");
  std::fprintf(f, "%u %u %llu\n", m.rows, m.cols, (unsigned long long)m.nnz);
  for (uint32_t r = 0; r < m.rows; ++r)
    for (uint32_t k = rp[r]; k < rp[r + 1]; ++k)
      std::fprintf(f, "%ld %ld %.*g\n", (long)r + index_base, (long)ci[k] + index_base, prec, v[k]);
  const bool ok = std::ferror(f) == 0;
  std::fclose(f);
  require(ok, VCLGB_GENERIC_FAILURE, "write error");
}

}  // namespace vclgb
