// io.cpp — the reference's on-disk matrix formats.
//
// smat_read_mtx reads MatrixMarket coordinate files the way the SpMM
// harness's reader does (src/cuda_hgemm/src/common/mmio_highlevel.h:514-680):
// rows padded up to a multiple of 16 and columns to a multiple of the block
// width; entries of a row kept in file order (not sorted); symmetric and
// hermitian files expanded by mirroring every off-diagonal entry, with the
// mirrored copy placed right after the entry in the fill order; complex files
// keep the real part; pattern files read as 1.0; duplicates kept. Values are
// returned as the doubles parsed from the file, so FP16 conversion happens
// once, as in the reference.
//
// smat_read_el reads the preprocessing tool's edge lists
// (preprocess/src/general/csr.cpp:166-290): leading '#' or '%' lines are
// skipped, each line is "row col [value]" split on single spaces, rows must
// come in ascending order (missing rows are empty), the column count is the
// largest column index + 1 and values are FP32.
//
// smat_write_el writes a matrix, optionally with its rows permuted, as the
// pattern-only edge list Matrix_Blocking saves as *_reordered.el
// (csr.cpp:150-161, test/general/Matrix_Blocking.cpp:42-49).
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "smat_internal.h"

namespace smat {
namespace {

struct FileCloser {
  FILE* f;
  ~FileCloser() {
    if (f) std::fclose(f);
  }
};

template <typename T>
T* dup_array(const std::vector<T>& v) {
  T* p = static_cast<T*>(std::malloc(std::max<size_t>(v.size(), 1) * sizeof(T)));
  if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
  return p;
}

// Reads the next whitespace-separated token; false at end of file.
bool next_token(FILE* f, std::string& tok) {
  tok.clear();
  int c;
  while ((c = std::fgetc(f)) != EOF && std::isspace(c)) {
  }
  if (c == EOF) return false;
  do {
    tok.push_back((char)c);
  } while ((c = std::fgetc(f)) != EOF && !std::isspace(c));
  return true;
}

bool parse_i64(const std::string& s, int64_t& v) {
  if (s.empty()) return false;
  errno = 0;
  char* end = nullptr;
  const long long x = std::strtoll(s.c_str(), &end, 10);
  if (errno || *end) return false;
  v = x;
  return true;
}

bool parse_f64(const std::string& s, double& v) {
  if (s.empty()) return false;
  errno = 0;
  char* end = nullptr;
  v = std::strtod(s.c_str(), &end);
  return !*end;
}

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

smat_status finish(smat_csr_file* out, int64_t rows, int64_t cols, const std::vector<int64_t>& rp,
                   const std::vector<int32_t>& ci, const void* vals, size_t val_bytes, int32_t dtype,
                   int32_t symmetric) {
  int64_t* prp = dup_array(rp);
  int32_t* pci = dup_array(ci);
  void* pv = nullptr;
  if (vals) {
    pv = std::malloc(std::max<size_t>(val_bytes, 1));
    if (pv && val_bytes) std::memcpy(pv, vals, val_bytes);
  }
  if (!prp || !pci || (vals && !pv)) {
    std::free(prp);
    std::free(pci);
    std::free(pv);
    return fail(SMAT_ERR_NOMEM, "out of host memory");
  }
  out->csr.rows = rows;
  out->csr.cols = cols;
  out->csr.nnz = (int64_t)ci.size();
  out->csr.row_ptr = prp;
  out->csr.col_idx = pci;
  out->csr.values = pv;
  out->csr.values_dtype = dtype;
  out->symmetric = symmetric;
  return SMAT_OK;
}

}  // namespace
}  // namespace smat

using namespace smat;

extern "C" {

smat_status smat_read_mtx(const char* path, int32_t col_pad, smat_csr_file* out) {
  if (!path || !out) return fail(SMAT_ERR_INVALID, "null argument");
  std::memset(out, 0, sizeof(*out));
  if (col_pad < 1) return fail(SMAT_ERR_INVALID, "col_pad must be >= 1");
  FileCloser fc{std::fopen(path, "r")};
  if (!fc.f) return fail(SMAT_ERR_INVALID, std::string("cannot open ") + path);
  FILE* f = fc.f;
  // banner: %%MatrixMarket matrix coordinate <field> <symmetry>
  char line[1030];
  if (!std::fgets(line, sizeof(line), f)) return fail(SMAT_ERR_INVALID, "empty MatrixMarket file");
  char b0[64] = {0}, b1[64] = {0}, b2[64] = {0}, b3[64] = {0}, b4[64] = {0};
  if (std::sscanf(line, "%63s %63s %63s %63s %63s", b0, b1, b2, b3, b4) != 5 ||
      std::string(b0) != "%%MatrixMarket")
    return fail(SMAT_ERR_INVALID, "bad MatrixMarket banner");
  const std::string obj = lower(b1), fmt = lower(b2), field = lower(b3), sym = lower(b4);
  if (obj != "matrix" || fmt != "coordinate")
    return fail(SMAT_ERR_UNSUPPORTED, "only coordinate matrices are supported");
  const bool is_pattern = field == "pattern", is_complex = field == "complex", is_int = field == "integer";
  if (!is_pattern && !is_complex && !is_int && field != "real" && field != "double")
    return fail(SMAT_ERR_INVALID, "unknown MatrixMarket field " + field);
  if (sym != "general" && sym != "symmetric" && sym != "hermitian" && sym != "skew-symmetric")
    return fail(SMAT_ERR_INVALID, "unknown MatrixMarket symmetry " + sym);
  const bool mirror = sym == "symmetric" || sym == "hermitian";
  // size line after comments
  int64_t m = 0, n = 0, nz = 0;
  for (;;) {
    if (!std::fgets(line, sizeof(line), f)) return fail(SMAT_ERR_INVALID, "missing size line");
    if (line[0] == '%') continue;
    long long a, b, c;
    if (std::sscanf(line, "%lld %lld %lld", &a, &b, &c) != 3) continue;  // blank line
    m = a;
    n = b;
    nz = c;
    break;
  }
  if (m < 0 || n < 0 || nz < 0 || m >= INT32_MAX || n >= INT32_MAX)
    return fail(SMAT_ERR_INVALID, "bad MatrixMarket size line");
  // padding (mmio_highlevel.h:514-520): rows to 16, columns to col_pad
  const int64_t mp = (m + 15) / 16 * 16;
  const int64_t np = (n + col_pad - 1) / col_pad * col_pad;
  std::vector<int64_t> ri(nz), cj(nz);
  std::vector<double> v(nz);
  std::string tok;
  for (int64_t i = 0; i < nz; i++) {
    int64_t a, b;
    if (!next_token(f, tok) || !parse_i64(tok, a) || !next_token(f, tok) || !parse_i64(tok, b))
      return fail(SMAT_ERR_INVALID, "truncated or malformed entry " + std::to_string(i));
    if (a < 1 || a > m || b < 1 || b > n)
      return fail(SMAT_ERR_INVALID, "entry " + std::to_string(i) + " out of range");
    double x = 1.0;
    if (!is_pattern) {
      if (!next_token(f, tok)) return fail(SMAT_ERR_INVALID, "missing value");
      if (is_int) {
        int64_t iv;
        if (!parse_i64(tok, iv)) return fail(SMAT_ERR_INVALID, "bad integer value");
        x = (double)iv;
      } else if (!parse_f64(tok, x)) {
        return fail(SMAT_ERR_INVALID, "bad value");
      }
      double imag = 0.0;  // read and dropped: the reference keeps the real part
      if (is_complex && (!next_token(f, tok) || !parse_f64(tok, imag)))
        return fail(SMAT_ERR_INVALID, "bad imaginary part");
    }
    ri[i] = a - 1;
    cj[i] = b - 1;
    v[i] = x;
  }
  // counts, then fill in entry order (mirrored copy right after its entry)
  std::vector<int64_t> rp(mp + 1, 0);
  for (int64_t i = 0; i < nz; i++) {
    rp[ri[i] + 1]++;
    if (mirror && ri[i] != cj[i]) rp[cj[i] + 1]++;
  }
  for (int64_t r = 0; r < mp; r++) rp[r + 1] += rp[r];
  std::vector<int64_t> fill(rp.begin(), rp.end() - 1);
  std::vector<int32_t> ci(rp[mp]);
  std::vector<double> vv(rp[mp]);
  for (int64_t i = 0; i < nz; i++) {
    int64_t o = fill[ri[i]]++;
    ci[o] = (int32_t)cj[i];
    vv[o] = v[i];
    if (mirror && ri[i] != cj[i]) {
      o = fill[cj[i]]++;
      ci[o] = (int32_t)ri[i];
      vv[o] = v[i];
    }
  }
  return finish(out, mp, np, rp, ci, vv.data(), vv.size() * sizeof(double), SMAT_F64, mirror ? 1 : 0);
}

smat_status smat_read_el(const char* path, int32_t pattern_only, smat_csr_file* out) {
  if (!path || !out) return fail(SMAT_ERR_INVALID, "null argument");
  std::memset(out, 0, sizeof(*out));
  FileCloser fc{std::fopen(path, "r")};
  if (!fc.f) return fail(SMAT_ERR_INVALID, std::string("cannot open ") + path);
  FILE* f = fc.f;
  std::vector<int64_t> rp(1, 0);
  std::vector<int32_t> ci;
  std::vector<float> vals;
  int64_t cur = -1, maxcol = 0, lineno = 0;
  bool header = true;
  std::string s;
  int c;
  for (;;) {
    s.clear();
    while ((c = std::fgetc(f)) != EOF && c != '\n') s.push_back((char)c);
    if (c == EOF && s.empty()) break;
    ++lineno;
    if (header && !s.empty() && (s[0] == '#' || s[0] == '%')) continue;
    header = false;
    // "row col [value]" on single spaces
    const size_t p1 = s.find(' ');
    if (p1 == std::string::npos) return fail(SMAT_ERR_INVALID, "malformed line " + std::to_string(lineno));
    const size_t p2 = s.find(' ', p1 + 1);
    int64_t r, col;
    if (!parse_i64(s.substr(0, p1), r) ||
        !parse_i64(s.substr(p1 + 1, p2 == std::string::npos ? std::string::npos : p2 - p1 - 1), col) || r < 0 ||
        col < 0 || col >= INT32_MAX)
      return fail(SMAT_ERR_INVALID, "malformed line " + std::to_string(lineno));
    float x = 1.0f;
    if (!pattern_only) {
      if (p2 == std::string::npos) return fail(SMAT_ERR_INVALID, "missing value on line " + std::to_string(lineno));
      const size_t p3 = s.find(' ', p2 + 1);
      const std::string vs = s.substr(p2 + 1, p3 == std::string::npos ? std::string::npos : p3 - p2 - 1);
      char* end = nullptr;
      errno = 0;
      x = std::strtof(vs.c_str(), &end);
      if (vs.empty() || *end) return fail(SMAT_ERR_INVALID, "bad value on line " + std::to_string(lineno));
    }
    if (r < cur) return fail(SMAT_ERR_INVALID, "edge list rows must be in ascending order");
    while (cur < r) {
      if (cur >= 0) rp.push_back((int64_t)ci.size());
      cur++;
    }
    ci.push_back((int32_t)col);
    if (!pattern_only) vals.push_back(x);
    maxcol = std::max(maxcol, col);
  }
  if (cur >= 0) rp.push_back((int64_t)ci.size());
  const int64_t rows = cur + 1;
  return finish(out, rows, rows > 0 ? maxcol + 1 : 0, rp, ci, pattern_only ? nullptr : vals.data(),
                vals.size() * sizeof(float), SMAT_F32, 0);
}

smat_status smat_write_el(const char* path, const smat_csr* A, const int64_t* row_perm) {
  if (!path || !A || !A->row_ptr || (A->nnz > 0 && !A->col_idx)) return fail(SMAT_ERR_INVALID, "null argument");
  FileCloser fc{std::fopen(path, "w")};
  if (!fc.f) return fail(SMAT_ERR_INVALID, std::string("cannot create ") + path);
  for (int64_t i = 0; i < A->rows; i++) {
    const int64_t r = row_perm ? row_perm[i] : i;
    if (r < 0 || r >= A->rows) return fail(SMAT_ERR_INVALID, "row_perm out of range");
    for (int64_t k = A->row_ptr[r]; k < A->row_ptr[r + 1]; k++)
      if (std::fprintf(fc.f, "%lld %d\n", (long long)i, A->col_idx[k]) < 0)
        return fail(SMAT_ERR_INVALID, "write failed");
  }
  return SMAT_OK;
}

smat_status smat_csr_file_free(smat_csr_file* f) {
  if (!f) return SMAT_OK;
  std::free(const_cast<int64_t*>(f->csr.row_ptr));
  std::free(const_cast<int32_t*>(f->csr.col_idx));
  std::free(const_cast<void*>(f->csr.values));
  std::memset(f, 0, sizeof(*f));
  return SMAT_OK;
}

}  // extern "C"
