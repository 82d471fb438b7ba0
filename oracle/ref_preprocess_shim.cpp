// ref_preprocess_shim.cpp — TEST INFRASTRUCTURE ONLY.
//
// A C-ABI wrapper around the reference's own preprocess code, compiled together
// with the reference sources (preprocess/src/general/*.cpp) by oracle/Makefile
// into oracle/_ref/libsmat_ref_preprocess.so. It builds the reference's CSR
// struct (preprocess/include/matrices.h:10-86) in memory and calls the
// reference functions unchanged. Used only by tests to pin the oracle and to
// generate golden fixtures.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <vector>

#include "blocking.h"
#include "matrices.h"
#include "utilities.h"

namespace {

// The reference CSR has no default constructor; build one field by field so
// that its destructor (csr.cpp:17-42) frees what we allocate here.
CSR* make_csr(int64_t rows, int64_t cols, const int64_t* rowptr, const int64_t* colidx,
              const float* val) {
  void* mem = ::operator new(sizeof(CSR));
  std::memset(mem, 0, sizeof(CSR));
  CSR* c = reinterpret_cast<CSR*>(mem);
  c->rows = rows;
  c->cols = cols;
  c->pattern_only = (val == nullptr);
  c->nzcount = new intT[rows];
  c->ja = new intT*[rows];
  c->ma = val ? new DataT*[rows] : nullptr;
  for (int64_t i = 0; i < rows; i++) {
    intT n = rowptr[i + 1] - rowptr[i];
    c->nzcount[i] = n;
    c->ja[i] = new intT[n];
    for (intT k = 0; k < n; k++) c->ja[i][k] = colidx[rowptr[i] + k];
    if (val) {
      c->ma[i] = new DataT[n];
      for (intT k = 0; k < n; k++) c->ma[i][k] = val[rowptr[i] + k];
    }
  }
  return c;
}

void free_csr(CSR* c) {
  if (c->ma) {
    for (intT i = 0; i < c->rows; i++) delete[] c->ma[i];
    delete[] c->ma;
    c->ma = nullptr;
  }
  c->pattern_only = true;  // ma already released above
  c->clean();
  delete[] c->ja;
  ::operator delete(c);
}

}  // namespace

extern "C" {

float ref_jaccard_group(const int64_t* a, int64_t na, int64_t ga, const int64_t* b, int64_t nb,
                        int64_t gb, int64_t bs) {
  std::vector<intT> A(a, a + na);
  return JaccardDistanceGroup(A, ga, (intT*)b, nb, gb, bs);
}

float ref_hamming_group(const int64_t* a, int64_t na, int64_t ga, const int64_t* b, int64_t nb,
                        int64_t gb, int64_t bs) {
  std::vector<intT> A(a, a + na);
  return HammingDistanceGroup(A, ga, (intT*)b, nb, gb, bs);
}

int64_t ref_merge_rows(const int64_t* a, int64_t na, const int64_t* b, int64_t nb, int64_t* out) {
  std::vector<intT> A(a, a + na);
  std::vector<intT> r = merge_rows(A, (intT*)b, nb);
  for (size_t i = 0; i < r.size(); i++) out[i] = r[i];
  return (int64_t)r.size();
}

// BlockingEngine::GetGrouping (blocking.cpp:616-657) with the settings of
// `Matrix_Blocking -a algo -b col_block -B row_block -F force_fixed -t tau`,
// then get_permutation (utilities.cpp:8-20) as CSR::reorder uses it.
// stats: [comparisons, merges, VBR_nzcount, VBR_nzblocks_count, VBR_longest_row]
void ref_reorder(int64_t rows, int64_t cols, const int64_t* rowptr, const int64_t* colidx,
                 float tau, int64_t col_block, int64_t row_block, int algo, int force_fixed,
                 int64_t* grouping_out, int64_t* perm_out, int64_t* stats) {
  CSR* c = make_csr(rows, cols, rowptr, colidx, nullptr);
  BlockingEngine be;
  be.tau = tau;
  be.col_block_size = col_block;
  be.row_block_size = row_block;
  be.use_groups = false;
  be.use_pattern = true;
  be.force_fixed_size = force_fixed != 0;
  be.blocking_algo = (BlockingType)algo;
  be.comparator = JaccardDistanceGroup;
  std::vector<intT> g = be.GetGrouping(*c);
  be.CollectBlockingInfo(*c);
  std::vector<intT> p = get_permutation(g);
  for (int64_t i = 0; i < rows; i++) {
    grouping_out[i] = g[i];
    perm_out[i] = p[i];
  }
  if (stats) {
    stats[0] = be.comparison_counter;
    stats[1] = be.merge_counter;
    stats[2] = be.VBR_nzcount;
    stats[3] = be.VBR_nzblocks_count;
    stats[4] = be.VBR_longest_row;
  }
  free_csr(c);
}

// CSR::read_from_edgelist (csr.cpp:166-290) with Matrix_Blocking's defaults
// (space delimiter, edge-list format, no symmetrisation). Returns the row
// count (or -1 if the reference threw); the outputs are malloc'd arrays the
// caller releases with ref_pre_free.
int64_t ref_read_el(const char* path, int pattern_only, int64_t* cols, int64_t** rowptr, int64_t** colidx,
                    float** val) {
  void* mem = ::operator new(sizeof(CSR));
  std::memset(mem, 0, sizeof(CSR));
  CSR* c = reinterpret_cast<CSR*>(mem);
  std::ifstream in(path);
  try {
    c->read_from_edgelist(in, " ", pattern_only != 0, el, false);
  } catch (...) {
    ::operator delete(mem);
    return -1;
  }
  int64_t nnz = 0;
  for (intT i = 0; i < c->rows; i++) nnz += c->nzcount[i];
  *cols = c->cols;
  *rowptr = static_cast<int64_t*>(std::malloc((c->rows + 1) * sizeof(int64_t)));
  *colidx = static_cast<int64_t*>(std::malloc(std::max<int64_t>(nnz, 1) * sizeof(int64_t)));
  *val = static_cast<float*>(std::malloc(std::max<int64_t>(nnz, 1) * sizeof(float)));
  int64_t p = 0;
  (*rowptr)[0] = 0;
  for (intT i = 0; i < c->rows; i++) {
    for (intT k = 0; k < c->nzcount[i]; k++) {
      (*colidx)[p] = c->ja[i][k];
      (*val)[p] = pattern_only ? 1.0f : c->ma[i][k];
      p++;
    }
    (*rowptr)[i + 1] = p;
  }
  const int64_t rows = c->rows;
  free_csr(c);
  return rows;
}

void ref_pre_free(void* p) { std::free(p); }

// CSR::multiply (csr.cpp:47-63) on a CSR built in memory: B and C column-major
// with leading dimension `rows`; C is accumulated in place.
void ref_csr_multiply(int64_t rows, int64_t cols, const int64_t* rowptr, const int64_t* colidx,
                      const float* val, float* B, int64_t b_cols, float* C) {
  CSR* c = make_csr(rows, cols, rowptr, colidx, val);
  c->multiply(B, b_cols, C);
  free_csr(c);
}

// CSR::reorder (csr.cpp:97-105) applied to a weighted CSR: returns the
// permuted rows' column indices and values in the output arrays.
void ref_csr_reorder_rows(int64_t rows, int64_t cols, const int64_t* rowptr,
                          const int64_t* colidx, const float* val, const int64_t* grouping,
                          int64_t* rowptr_out, int64_t* colidx_out, float* val_out) {
  CSR* c = make_csr(rows, cols, rowptr, colidx, val);
  std::vector<intT> g(grouping, grouping + rows);
  c->reorder(g);
  int64_t p = 0;
  rowptr_out[0] = 0;
  for (int64_t i = 0; i < rows; i++) {
    for (intT k = 0; k < c->nzcount[i]; k++) {
      colidx_out[p] = c->ja[i][k];
      val_out[p] = c->ma[i][k];
      p++;
    }
    rowptr_out[i + 1] = p;
  }
  free_csr(c);
}

}  // extern "C"
