// Matrix Market exchange files for CompRowMatrix and DenseVector, as MTJ
// reads and writes them (mtj/src/no/uib/cipr/matrix/io/MatrixVectorReader.java,
// MatrixVectorWriter.java, MatrixInfo.java:239-273, VectorInfo.java:162-184):
//
// * reading follows CompRowMatrix(MatrixVectorReader)
//   (sparse/CompRowMatrix.java:68-146): an optional "%%MatrixMarket matrix
//   coordinate <field> <symmetry>" header (real general when absent), '%'
//   comments anywhere after it, whitespace-separated tokens; the pattern of
//   each row is the set of its columns, sorted; values are stored in file
//   order (a repeated entry keeps the last value); symmetric files add the
//   mirrored entries afterwards, skew-symmetric files the negated ones;
//   pattern, complex and array (dense) matrices are rejected;
// * DenseVector(MatrixVectorReader) (DenseVector.java:52-96): array or
//   coordinate vectors, real or integer;
// * writing prints what MatrixVectorWriter prints: the header line, the size
//   line ("%10d %10d %19d" for a coordinate matrix, "%10d" for an array
//   vector) and one entry per line ("%10d %10d % .12e", 1-based, row by row
//   in CSR order; "% .12e" for vector entries).
//
// Numbers are parsed with strtod, which rounds correctly, as
// Double.parseDouble does.  Java's Formatter rounds the shortest decimal
// representation of a double half-up to 13 digits, C's printf the exact
// binary value half-even; the two can differ in the 13th digit of a value
// that lies on a rounding tie.  Host code only: the files are read and
// written through the C library.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "common.cuh"

namespace {

// The tokenizer of MatrixVectorReader: whitespace is ' ' and \t..\r (0x09 to
// 0x0e), '%' starts a comment to the end of the line, every other byte is
// part of a word.
struct Tokens {
  std::string text;
  size_t pos = 0;
  bool next(std::string& w) {
    for (;;) {
      while (pos < text.size() && (text[pos] == ' ' || (text[pos] >= 0x09 && text[pos] <= 0x0e))) ++pos;
      if (pos >= text.size()) return false;
      if (text[pos] == '%') {
        while (pos < text.size() && text[pos] != '\n' && text[pos] != '\r') ++pos;
        continue;
      }
      break;
    }
    const size_t b = pos;
    while (pos < text.size() && text[pos] != '%' && !(text[pos] == ' ' || (text[pos] >= 0x09 && text[pos] <= 0x0e)))
      ++pos;
    w.assign(text, b, pos - b);
    return true;
  }
};

struct MMError {
  rsg_status st;
};

bool read_file(const char* path, std::string& out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, k);
  std::fclose(f);
  return true;
}

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// Integer.parseInt
int parse_int(const std::string& w) {
  if (w.empty()) throw MMError{RSG_BAD_ARG};
  size_t i = (w[0] == '-' || w[0] == '+') ? 1 : 0;
  if (i == w.size()) throw MMError{RSG_BAD_ARG};
  long long v = 0;
  for (; i < w.size(); ++i) {
    if (w[i] < '0' || w[i] > '9') throw MMError{RSG_BAD_ARG};
    v = v * 10 + (w[i] - '0');
    if (v > 2147483648LL) throw MMError{RSG_BAD_ARG};
  }
  if (w[0] == '-') v = -v;
  if (v > 2147483647LL || v < -2147483648LL) throw MMError{RSG_BAD_ARG};
  return (int)v;
}

// Double.parseDouble on a word (the tokenizer lower-cases words; an
// optional d/f suffix allowed)
double parse_double(std::string w) {
  w = lower(w);
  if (!w.empty() && (w.back() == 'd' || w.back() == 'f') && w.size() > 1 &&
      (std::isdigit((unsigned char)w[w.size() - 2]) || w[w.size() - 2] == '.'))
    w.pop_back();
  if (w == "nan" || w == "+nan" || w == "-nan") return NAN;
  if (w == "infinity" || w == "+infinity") return INFINITY;
  if (w == "-infinity") return -INFINITY;
  if (w.empty() || w.find_first_not_of("0123456789+-.e") != std::string::npos) throw MMError{RSG_BAD_ARG};
  char* end = nullptr;
  errno = 0;
  const double v = std::strtod(w.c_str(), &end);
  if (end != w.c_str() + w.size()) throw MMError{RSG_BAD_ARG};
  return v;
}

struct Header {
  bool present = false, sparse = true;
  std::string field = "real", symmetry = "general";
};

// hasInfo + readMatrixInfo / readVectorInfo: the first line, split on spaces
Header read_header(Tokens& t, bool matrix) {
  Header h;
  const std::string& s = t.text;
  size_t e = s.find('\n');
  std::string line = s.substr(0, e == std::string::npos ? s.size() : e);
  while (!line.empty() && (line.back() == '\r' || line.back() == ' ' || line.back() == '\t')) line.pop_back();
  size_t b = line.find_first_not_of(" \t");
  line = b == std::string::npos ? "" : line.substr(b);
  std::vector<std::string> c;
  for (size_t i = 0; i < line.size();) {
    size_t j = line.find(' ', i);
    if (j == std::string::npos) j = line.size();
    if (j > i) c.push_back(lower(line.substr(i, j - i)));
    i = j + 1;
  }
  if (c.empty() || c[0] != "%%matrixmarket") return h;
  h.present = true;
  if (c.size() != (matrix ? 5u : 4u) || c[1] != (matrix ? "matrix" : "vector")) throw MMError{RSG_BAD_ARG};
  if (c[2] == "coordinate") h.sparse = true;
  else if (c[2] == "array") h.sparse = false;
  else throw MMError{RSG_BAD_ARG};
  if (c[3] != "real" && c[3] != "integer" && c[3] != "complex" && c[3] != "pattern") throw MMError{RSG_BAD_ARG};
  h.field = c[3];
  if (matrix) {
    if (c[4] != "general" && c[4] != "symmetric" && c[4] != "skew-symmetric" && c[4] != "hermitian")
      throw MMError{RSG_BAD_ARG};
    h.symmetry = c[4];
  }
  t.pos = e == std::string::npos ? s.size() : e + 1;
  return h;
}

struct Coo {
  int rows = 0, cols = 0;
  std::vector<int> rp, col;
  std::vector<double> val;
};

// CompRowMatrix(MatrixVectorReader)
Coo read_matrix(const char* path) {
  Tokens t;
  if (!path || !read_file(path, t.text)) throw MMError{RSG_BAD_ARG};
  const Header h = read_header(t, true);
  if (h.field == "pattern" || h.field == "complex" || !h.sparse) throw MMError{RSG_UNSUPPORTED};
  if (h.symmetry == "hermitian") throw MMError{RSG_UNSUPPORTED};
  std::string w;
  auto next_int = [&] {
    if (!t.next(w)) throw MMError{RSG_BAD_ARG};
    return parse_int(w);
  };
  Coo m;
  m.rows = next_int();
  m.cols = next_int();
  const int ne = next_int();
  if (m.rows < 0 || m.cols < 0 || ne < 0) throw MMError{RSG_BAD_ARG};
  std::vector<int> r(ne), c(ne);
  std::vector<double> v(ne);
  for (int i = 0; i < ne; ++i) {
    r[i] = next_int() - 1;
    c[i] = next_int() - 1;
    if (!t.next(w)) throw MMError{RSG_BAD_ARG};
    v[i] = parse_double(w);
    if (r[i] < 0 || r[i] >= m.rows || c[i] < 0 || c[i] >= m.cols) throw MMError{RSG_BAD_ARG};
  }
  const bool sym = h.symmetry == "symmetric", skew = h.symmetry == "skew-symmetric";
  std::vector<std::vector<int>> nz(m.rows);
  for (int i = 0; i < ne; ++i) nz[r[i]].push_back(c[i]);
  if (sym || skew)
    for (int i = 0; i < ne; ++i)
      if (r[i] != c[i]) {
        if (c[i] >= m.rows || r[i] >= m.cols) throw MMError{RSG_BAD_ARG};
        nz[c[i]].push_back(r[i]);
      }
  m.rp.assign(m.rows + 1, 0);
  for (int i = 0; i < m.rows; ++i) {
    auto& z = nz[i];
    std::sort(z.begin(), z.end());
    z.erase(std::unique(z.begin(), z.end()), z.end());
    m.rp[i + 1] = m.rp[i] + (int)z.size();
  }
  m.col.reserve(m.rp[m.rows]);
  for (auto& z : nz) m.col.insert(m.col.end(), z.begin(), z.end());
  m.val.assign(m.col.size(), 0.0);
  auto set = [&](int i, int j, double x) {
    const auto b = m.col.begin() + m.rp[i], e = m.col.begin() + m.rp[i + 1];
    m.val[std::lower_bound(b, e, j) - m.col.begin()] = x;
  };
  for (int i = 0; i < ne; ++i) set(r[i], c[i], v[i]);
  if (sym || skew)
    for (int i = 0; i < ne; ++i)
      if (r[i] != c[i]) set(c[i], r[i], skew ? -v[i] : v[i]);
  return m;
}

// DenseVector(MatrixVectorReader)
std::vector<double> read_vector(const char* path) {
  Tokens t;
  if (!path || !read_file(path, t.text)) throw MMError{RSG_BAD_ARG};
  const Header h = read_header(t, false);  // no header: new VectorInfo(true, Real), a coordinate vector
  if (h.field == "pattern" || h.field == "complex") throw MMError{RSG_UNSUPPORTED};
  std::string w;
  auto next = [&] {
    if (!t.next(w)) throw MMError{RSG_BAD_ARG};
    return w;
  };
  const int n = parse_int(next());
  if (n < 0) throw MMError{RSG_BAD_ARG};
  std::vector<double> x(n, 0.0);
  if (h.sparse) {
    const int ne = parse_int(next());
    if (ne < 0) throw MMError{RSG_BAD_ARG};
    std::vector<int> idx(ne);
    std::vector<double> v(ne);
    for (int i = 0; i < ne; ++i) {
      idx[i] = parse_int(next()) - 1;
      v[i] = parse_double(next());
      if (idx[i] < 0 || idx[i] >= n) throw MMError{RSG_BAD_ARG};
    }
    for (int i = 0; i < ne; ++i) x[idx[i]] = v[i];
  } else {
    for (int i = 0; i < n; ++i) x[i] = parse_double(next());
  }
  return x;
}

// "% .12e" of java.util.Formatter for the special values, printf otherwise
void put_e12(FILE* f, double v) {
  if (std::isnan(v)) std::fputs("NaN", f);
  else if (std::isinf(v)) std::fputs(v > 0 ? " Infinity" : "-Infinity", f);
  else std::fprintf(f, "% .12e", v);
}

template <typename F>
rsg_status mm_guard(F&& f) {
  try {
    f();
    return RSG_OK;
  } catch (const MMError& e) {
    return e.st;
  } catch (...) {
    return RSG_BAD_ARG;
  }
}

}  // namespace

extern "C" {

rsg_status rsg_mm_read_matrix_size(const char* path, int32_t* rows, int32_t* cols, int64_t* nnz) {
  if (!path || !rows || !cols || !nnz) return RSG_BAD_ARG;
  return mm_guard([&] {
    const Coo m = read_matrix(path);
    *rows = m.rows;
    *cols = m.cols;
    *nnz = (int64_t)m.col.size();
  });
}

rsg_status rsg_mm_read_csr(const char* path, int32_t rows, int64_t nnz, int32_t* row_ptr, int32_t* col, double* val) {
  if (!path || !row_ptr || (nnz > 0 && (!col || !val))) return RSG_BAD_ARG;
  return mm_guard([&] {
    const Coo m = read_matrix(path);
    if (m.rows != rows || (int64_t)m.col.size() != nnz) throw MMError{RSG_BAD_ARG};
    std::copy(m.rp.begin(), m.rp.end(), row_ptr);
    std::copy(m.col.begin(), m.col.end(), col);
    std::copy(m.val.begin(), m.val.end(), val);
  });
}

rsg_status rsg_mm_write_csr(const char* path, int32_t rows, int32_t cols, const int32_t* row_ptr, const int32_t* col,
                            const double* val) {
  if (!path || rows < 0 || cols < 0 || !row_ptr) return RSG_BAD_ARG;
  const int64_t nnz = row_ptr[rows];
  if (nnz > 0 && (!col || !val)) return RSG_BAD_ARG;
  for (int i = 0; i < rows; ++i)
    if (row_ptr[i + 1] < row_ptr[i]) return RSG_BAD_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return RSG_BAD_ARG;
  std::fputs("%%MatrixMarket matrix coordinate real general\n", f);
  std::fprintf(f, "%10d %10d %19lld\n", rows, cols, (long long)nnz);
  for (int i = 0; i < rows; ++i)
    for (int q = row_ptr[i]; q < row_ptr[i + 1]; ++q) {
      std::fprintf(f, "%10d %10d ", i + 1, col[q] + 1);
      put_e12(f, val[q]);
      std::fputc('\n', f);
    }
  return std::fclose(f) == 0 ? RSG_OK : RSG_BAD_ARG;
}

rsg_status rsg_mm_read_vector_size(const char* path, int32_t* size) {
  if (!path || !size) return RSG_BAD_ARG;
  return mm_guard([&] { *size = (int32_t)read_vector(path).size(); });
}

rsg_status rsg_mm_read_vector(const char* path, int32_t size, double* x) {
  if (!path || (size > 0 && !x)) return RSG_BAD_ARG;
  return mm_guard([&] {
    const std::vector<double> v = read_vector(path);
    if ((int32_t)v.size() != size) throw MMError{RSG_BAD_ARG};
    std::copy(v.begin(), v.end(), x);
  });
}

rsg_status rsg_mm_write_vector(const char* path, int32_t size, const double* x) {
  if (!path || size < 0 || (size > 0 && !x)) return RSG_BAD_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return RSG_BAD_ARG;
  std::fputs("%%MatrixMarket vector array real\n", f);
  std::fprintf(f, "%10d\n", size);
  for (int i = 0; i < size; ++i) {
    put_e12(f, x[i]);
    std::fputc('\n', f);
  }
  return std::fclose(f) == 0 ? RSG_OK : RSG_BAD_ARG;
}

}  // extern "C"
