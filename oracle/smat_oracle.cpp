// smat_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference SMaT algorithms on the SpMM path, used as the
// checker by tests/, by __graft_entry__.smoke() and by bench.py's cpu_baseline
// leg. Nothing in the product library links or calls this file.
//
// Parity pinning: every function here is checked against the reference itself
// (oracle/_ref, compiled from the reference sources by oracle/Makefile) and
// against golden fixtures in tests/golden/ produced by that build
// (tests/golden/make_golden.py), plus the reference's own known-answer test
// for the Jaccard distance (preprocess/test/general/TEST_similarities.cpp).
//
// Reference citations are paths inside the ajit283/sptc-smat project.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <set>
#include <utility>
#include <vector>

namespace {

typedef long intT;  // preprocess/include/definitions.h:4

// preprocess/src/general/blocking.cpp:904-975 (JaccardDistanceGroup), with
// count_zeros = 1: a block column present on one side only adds the OTHER
// side's group size to `count`.
float jaccard_group(const intT* a, intT na, intT ga, const intT* b, intT nb, intT gb, intT bs) {
  if (na == 0 && nb == 0) return 0;
  if (na == 0 || nb == 0) return 1;
  const intT add_a = gb, add_b = ga;
  intT i = 0, j = 0, count = 0, blocks_a = 0, blocks_b = 0;
  while (i < na && j < nb) {
    intT pa = a[i] / bs, pb = b[j] / bs;
    if (pa < pb) {
      count += add_a; blocks_a++;
      while (i < na && a[i] / bs == pa) i++;
    } else if (pa > pb) {
      count += add_b; blocks_b++;
      while (j < nb && b[j] / bs == pb) j++;
    } else {
      blocks_a++; blocks_b++;
      while (i < na && a[i] / bs == pa) i++;
      while (j < nb && b[j] / bs == pb) j++;
    }
  }
  while (i < na) {
    intT pa = a[i] / bs;
    count += add_a; blocks_a++;
    while (i < na && a[i] / bs == pa) i++;
  }
  while (j < nb) {
    intT pb = b[j] / bs;
    count += add_b; blocks_b++;
    while (j < nb && b[j] / bs == pb) j++;
  }
  return (float)((2.0 * count) / (double)(blocks_a * ga + blocks_b * gb + count));
}

// preprocess/src/general/utilities.cpp:145-173 (merge_rows). Reproduces the
// reference exactly, including its early exit: once a B element lies beyond the
// remaining A range (or B runs out), the remaining A elements are NOT copied.
std::vector<intT> merge_rows(const std::vector<intT>& A, const intT* B, intT nb) {
  std::vector<intT> result;
  auto i = A.begin();
  intT j = 0;
  while (j < nb) {
    intT bv = B[j];
    auto ni = std::lower_bound(i, A.end(), bv);
    if (ni == A.end()) break;
    result.insert(result.end(), i, ni);
    result.push_back(bv);
    if (*ni == bv) ++ni;
    i = ni;
    j++;
  }
  result.insert(result.end(), B + j, B + nb);
  return result;
}

// preprocess/src/general/utilities.cpp:8-20 (get_permutation): std::sort of
// iota by group id. The sort is NOT stable; the tie order is that of
// libstdc++'s introsort, so this must be compiled against libstdc++ to agree.
std::vector<intT> get_permutation(const std::vector<intT>& grouping) {
  auto comp = [&](int i, int j) { return grouping[i] < grouping[j]; };
  std::vector<intT> v(grouping.size());
  std::iota(v.begin(), v.end(), 0);
  std::sort(v.begin(), v.end(), comp);
  return v;
}

// preprocess/src/general/utilities.cpp:45-54 (get_fixed_size_grouping).
std::vector<intT> fixed_size_grouping(const std::vector<intT>& grouping, intT row_block) {
  std::vector<intT> out(grouping.size(), -1);
  std::vector<intT> perm = get_permutation(grouping);
  for (intT i = 0; i < (intT)perm.size(); i++) out[perm[i]] = i / row_block;
  return out;
}

}  // namespace

extern "C" {

float orc_jaccard_group(const int64_t* a, int64_t na, int64_t ga, const int64_t* b, int64_t nb,
                        int64_t gb, int64_t bs) {
  return jaccard_group((const intT*)a, na, ga, (const intT*)b, nb, gb, bs);
}

// Returns the merged length; `out` must hold na + nb entries.
int64_t orc_merge_rows(const int64_t* a, int64_t na, const int64_t* b, int64_t nb, int64_t* out) {
  std::vector<intT> A(a, a + na);
  std::vector<intT> r = merge_rows(A, (const intT*)b, nb);
  std::copy(r.begin(), r.end(), out);
  return (int64_t)r.size();
}

// preprocess/src/general/blocking.cpp:431-547 (IterativeBlockingKeeper), as
// selected by `Matrix_Blocking -a 5` with the CLI defaults of
// preprocess/include/input.h:21-22 (use_pattern = 1; the group size passed
// to the distance is always the current group size, blocking.cpp:480).
// `rowptr/cols` is a CSR pattern (cols in file order per row).
// stats[0] = comparisons, stats[1] = merges.
void orc_keeper_grouping(int64_t rows, const int64_t* rowptr, const int64_t* cols, float tau,
                         int64_t col_block, int64_t max_row_block, int64_t* grouping_out,
                         int64_t* stats) {
  std::vector<intT> grouping(rows, -1);
  // `float distances[rows] = {-1}` is a GCC variable-length array with an
  // initialiser: element 0 is -1 and every other element is 0.
  std::vector<float> distances(rows, 0.0f);
  if (rows > 0) distances[0] = -1;
  intT comparisons = 0, merges = 0;
  for (intT i = 0; i < rows; i++) {
    if (grouping[i] != -1) continue;
    std::set<std::pair<float, intT>> best;
    std::vector<intT> merged;
    const intT group_number = i + rows;
    std::vector<intT> pattern(cols + rowptr[i], cols + rowptr[i + 1]);
    intT gsize = 1;
    grouping[i] = group_number;
    merged.push_back(i);
    for (intT j = i + 1; j < rows; j++) {
      if (gsize == max_row_block) break;
      if (distances[i] != -1 && distances[j] != -1 && std::fabs(distances[i] - distances[j]) > tau) {
        distances[j] = -1;
        continue;
      }
      if (grouping[j] == -1) {
        comparisons++;
        const intT* rj = (const intT*)(cols + rowptr[j]);
        intT nj = rowptr[j + 1] - rowptr[j];
        float d = jaccard_group(pattern.data(), (intT)pattern.size(), gsize, rj, nj, 1, col_block);
        distances[j] = d;
        if (d <= tau) {
          merges++;
          grouping[j] = group_number;
          merged.push_back(j);
          pattern = merge_rows(pattern, rj, nj);
          gsize++;
        } else {
          best.insert({d, j});
          size_t keep = (size_t)max_row_block - merged.size();
          if (best.size() > keep) {
            // blocking.cpp:507-509 starts the trim iterator at end() and
            // advances it `keep` times; with libstdc++'s red-black tree that
            // walks from the header node into the rightmost subtree, so the
            // set loses some of its LARGEST entries, not those past `keep`.
            auto it = best.end();
            std::advance(it, keep);
            best.erase(it, best.end());
          }
        }
      }
    }
    if (gsize < max_row_block) {
      for (auto it = best.begin(); it != best.end() && gsize != max_row_block; ++it) {
        grouping[it->second] = group_number;
        merged.push_back(it->second);
        gsize++;
      }
    }
    if (gsize == max_row_block)
      for (intT idx : merged) grouping[idx] -= rows;
  }
  std::copy(grouping.begin(), grouping.end(), (intT*)grouping_out);
  if (stats) { stats[0] = comparisons; stats[1] = merges; }
}

void orc_permutation(const int64_t* grouping, int64_t n, int64_t* perm_out) {
  std::vector<intT> g((const intT*)grouping, (const intT*)grouping + n);
  std::vector<intT> p = get_permutation(g);
  std::copy(p.begin(), p.end(), (intT*)perm_out);
}

void orc_fixed_size_grouping(const int64_t* grouping, int64_t n, int64_t row_block, int64_t* out) {
  std::vector<intT> g((const intT*)grouping, (const intT*)grouping + n);
  std::vector<intT> r = fixed_size_grouping(g, row_block);
  std::copy(r.begin(), r.end(), (intT*)out);
}

// The whole row-reordering step of `Matrix_Blocking -a 5 -b b -B B -F f -t tau`
// (preprocess/test/general/Matrix_Blocking.cpp:20,41; blocking.cpp:616-657;
// csr.cpp:97-105): grouping -> optional fixed-size regrouping -> permutation.
// New row r of the reordered matrix is old row perm_out[r] (utilities.h:96-104).
void orc_reorder(int64_t rows, const int64_t* rowptr, const int64_t* cols, float tau,
                 int64_t col_block, int64_t row_block, int force_fixed, int64_t* perm_out,
                 int64_t* grouping_out, int64_t* stats) {
  std::vector<intT> g(rows);
  orc_keeper_grouping(rows, rowptr, cols, tau, col_block, row_block, (int64_t*)g.data(), stats);
  if (force_fixed) g = fixed_size_grouping(g, row_block);
  if (grouping_out) std::copy(g.begin(), g.end(), (intT*)grouping_out);
  std::vector<intT> p = get_permutation(g);
  std::copy(p.begin(), p.end(), (intT*)perm_out);
}

// src/cuda_hgemm/src/common/matrix.h:666-792 (SparseMatrix::csrToBcsr),
// restated over the same dense block grid. Blocks are 16 x k. Two calls: the
// first (outputs NULL) returns nnzb; the second fills
//   bcsr_rowptr[rows/16 + 1], bcsr_colidx[nnzb] (column START, a multiple of k),
//   bcsr_val[nnzb * 16 * k] (fp16 bit patterns, row-major inside a block),
//   block_info[grid] (0 zero, 1 "2:4" by the reference heuristic, 2 dense).
// m_row must already be padded to a multiple of 16 and m_col to a multiple
// of k (mmio_highlevel.h:514-520).
int64_t orc_csr_to_bcsr(int64_t m_row, int64_t m_col, int k, const int32_t* rowptr,
                        const int32_t* colidx, const uint16_t* val, int32_t* bcsr_rowptr,
                        int32_t* bcsr_colidx, uint16_t* bcsr_val, int32_t* block_info) {
  const int64_t ncr = (m_col + k - 1) / k;
  const int64_t nrr = (m_row + 15) / 16;
  std::vector<int32_t> info(nrr * ncr, 0);
  int64_t nnzb = 0;
  for (int64_t row = 0; row < m_row; row++) {
    for (int64_t j = rowptr[row]; j < rowptr[row + 1]; j++) {
      int64_t col = colidx[j];
      int64_t bi = (row / 16) * ncr + col / k;
      if (info[bi] == 0) {
        info[bi] = 1;
        nnzb++;
      } else if (info[bi] == 1) {
        int64_t r24 = col % 4;
        if ((r24 == 2 || r24 == 3) && j >= rowptr[row] + 2 && colidx[j - 1] == col - 1 &&
            colidx[j - 2] == col - 2)
          info[bi] = 2;
      }
    }
  }
  if (!bcsr_rowptr) return nnzb;
  std::vector<int32_t> rel(nrr * ncr);
  int32_t r = 0;
  for (int64_t i = 0; i < nrr * ncr; i++) rel[i] = info[i] != 0 ? r++ : -1;
  int64_t nb = 0;
  for (int64_t row = 0; row < m_row; row += 16) {
    bcsr_rowptr[row / 16] = (int32_t)nb;
    for (int64_t col = 0; col < m_col; col += k) {
      if (info[(row / 16) * ncr + col / k] == 0) continue;
      bcsr_colidx[nb++] = (int32_t)col;
    }
  }
  bcsr_rowptr[m_row / 16] = (int32_t)nb;
  std::memset(bcsr_val, 0, sizeof(uint16_t) * nnzb * 16 * k);
  for (int64_t row = 0; row < m_row; row++) {
    for (int64_t j = rowptr[row]; j < rowptr[row + 1]; j++) {
      int64_t col = colidx[j];
      int64_t bi = (row / 16) * ncr + col / k;
      int64_t off = (row % 16) * k + col % k;
      bcsr_val[(int64_t)rel[bi] * 16 * k + off] = val[j];
    }
  }
  if (block_info) std::copy(info.begin(), info.end(), block_info);
  return nnzb;
}

// src/cuda_hgemm/src/common/matrix.h:794-1137 (SparseMatrix::bcsrBlocking):
// groups the 16 x k blocks of a BCSR (as csrToBcsr builds it) into merged
// TILES of 4 x 4 blocks (64 rows x 4k columns), restated with a map lookup
// in place of the reference's linear search over the tiles made so far
// (the keys are unique, so the result is the same). Reproduced as the
// reference has it:
//   * tiles are numbered in order of first appearance while walking the
//     blocks in BCSR order (:814-902), not sorted by column inside a tile row;
//   * a tile holds its 16 blocks block-major, each block row-major, at
//     k*4*(row offset) + 16*(column offset) (:851, :878-879);
//   * the tile row pointer gets one entry per NON-EMPTY tile row, plus the
//     final count (:932-958): tile rows without a tile get no entry;
//   * block_info / rel_map cover the full tile grid, rel_map numbers the
//     tiles in grid (row-major) order (:921-930);
//   * tile_info labels each of the 16 positions 0 (all zero) / 1 (no group
//     of four with more than two nonzeros) / 2, reading the tile's values as
//     a ROW-MAJOR 64 x 4k matrix (:1036-1088), which is not the layout they
//     were stored in.
// Two calls: with out_rowptr NULL it returns the tile count and sets
// *n_rowptr; the second fills rowptr[*n_rowptr], colidx[ntiles],
// val[ntiles * 256 * k], block_info / rel_map [tile rows * tile cols] and
// tile_info[ntiles * 16].
int64_t orc_bcsr_blocking(int64_t m_row, int64_t m_col, int k, int64_t nnzb, const int32_t* brp,
                          const int32_t* bci, const uint16_t* bval, int64_t* n_rowptr, int32_t* out_rowptr,
                          int32_t* out_colidx, uint16_t* out_val, int32_t* block_info, int32_t* rel_map,
                          int32_t* tile_info) {
  const int64_t tw = 4 * (int64_t)k, th = 64, tsz = 256 * (int64_t)k;
  const int64_t ncr = (m_col + tw - 1) / tw, nrr = (m_row + th - 1) / th;
  std::map<std::pair<int64_t, int64_t>, int64_t> tile_of;
  std::vector<int64_t> ty, tx;                   // tile row start / column start, by tile
  std::vector<std::vector<uint16_t>> tv;          // values, by tile
  int64_t br = 0;
  for (int64_t i = 0; i < nnzb; i++) {
    while (br < m_row / 16 && brp[br + 1] <= i) br++;
    const int64_t row = br * 16, col = bci[i];
    const int64_t y = row - row % th, x = col - col % tw;
    auto it = tile_of.find({y, x});
    int64_t t;
    if (it == tile_of.end()) {
      t = (int64_t)ty.size();
      tile_of[{y, x}] = t;
      ty.push_back(y);
      tx.push_back(x);
      tv.emplace_back(tsz, 0);
    } else {
      t = it->second;
    }
    const int64_t dst = 4 * (int64_t)k * (row - y) + 16 * (col - x);
    std::memcpy(tv[t].data() + dst, bval + i * 16 * (int64_t)k, sizeof(uint16_t) * 16 * k);
  }
  const int64_t nt = (int64_t)ty.size();
  std::vector<int32_t> rp;
  int64_t cur = -1;
  for (int64_t t = 0; t < nt; t++)
    if (ty[t] != cur) {
      cur = ty[t];
      rp.push_back((int32_t)t);
    }
  rp.push_back((int32_t)nt);
  if (n_rowptr) *n_rowptr = (int64_t)rp.size();
  if (!out_rowptr) return nt;
  std::copy(rp.begin(), rp.end(), out_rowptr);
  std::vector<int32_t> info(nrr * ncr, 0);
  for (int64_t t = 0; t < nt; t++) {
    out_colidx[t] = (int32_t)tx[t];
    std::memcpy(out_val + t * tsz, tv[t].data(), sizeof(uint16_t) * tsz);
    info[(ty[t] / th) * ncr + tx[t] / tw] = 1;
  }
  int32_t r = 0;
  for (int64_t g = 0; g < nrr * ncr; g++) {
    block_info[g] = info[g];
    rel_map[g] = info[g] ? r++ : -1;
  }
  for (int64_t t = 0; t < nt; t++)
    for (int sr = 0; sr < 4; sr++)
      for (int sc = 0; sc < 4; sc++) {
        bool any = false, two_four = true;
        for (int rr = 0; rr < 16; rr++) {
          const uint16_t* rowp = out_val + t * tsz + (int64_t)(sr * 16 + rr) * tw;
          for (int g = 0; g < k / 4; g++) {
            int nz = 0;
            for (int c = 0; c < 4; c++) nz += (rowp[sc * k + 4 * g + c] & 0x7fff) != 0;
            if (nz > 0) any = true;
            if (nz > 2) two_four = false;
          }
        }
        tile_info[t * 16 + sr * 4 + sc] = any ? (two_four ? 1 : 2) : 0;
      }
  return nt;
}

// Exact 2:4 predicate on one bh x bw block (row-major, fp16 bits; +0 and -0
// are zero): every aligned group of 4 columns in every row has at most 2
// nonzeros. Mirrors src/utils.py:163-174 (is_block_2_4), which flags a block
// as 2:4 unless some group holds more than 2 nonzeros.
int orc_is_block_24(const uint16_t* blk, int bh, int bw) {
  for (int r = 0; r < bh; r++)
    for (int g = 0; g < bw; g += 4) {
      int nz = 0;
      for (int c = g; c < g + 4; c++) nz += (blk[r * bw + c] & 0x7fff) != 0;
      if (nz > 2) return 0;
    }
  return 1;
}

// FP64 CPU product, the numerical oracle: C = A * B with A in CSR (double
// values). B element (k, n) is at B[k * ldb_k + n * ldb_n]; C element (i, n)
// is written to C[i * ldc_i + n * ldc_n].
void orc_spmm_f64(int64_t rows, int64_t n_cols, const int64_t* rowptr, const int64_t* colidx,
                  const double* val, const double* B, int64_t ldb_k, int64_t ldb_n, double* C,
                  int64_t ldc_i, int64_t ldc_n) {
  std::vector<double> acc(n_cols);
  for (int64_t i = 0; i < rows; i++) {
    std::fill(acc.begin(), acc.end(), 0.0);
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; p++) {
      const double v = val[p];
      const double* b = B + colidx[p] * ldb_k;
      for (int64_t n = 0; n < n_cols; n++) acc[n] += v * b[n * ldb_n];
    }
    for (int64_t n = 0; n < n_cols; n++) C[i * ldc_i + n * ldc_n] = acc[n];
  }
}

// preprocess/src/general/csr.cpp:47-63 (CSR::multiply), the reference's CPU
// SpMM: serial FP32, B and C column-major with leading dimension `rows`,
// C accumulated in place (the caller zeroes it).
void orc_csr_multiply_f32(int64_t rows, const int64_t* rowptr, const int64_t* colidx,
                          const float* val, const float* B, int64_t b_cols, float* C) {
  for (int64_t i = 0; i < rows; i++)
    for (int64_t nz = rowptr[i]; nz < rowptr[i + 1]; nz++) {
      int64_t col = colidx[nz];
      float v = val[nz];
      for (int64_t j = 0; j < b_cols; j++) C[i + j * rows] += v * B[col + j * rows];
    }
}

// CSR::multiply's loop (csr.cpp:47-63) restricted to rows [r0, r1) of a
// matrix whose B and C are column-major with leading dimension `ld`
// (the full row count, as in the reference). Used to time bounded samples
// and to split the rows over host threads.
void orc_csr_multiply_f32_range(int64_t ld, int64_t r0, int64_t r1, const int64_t* rowptr,
                                const int64_t* colidx, const float* val, const float* B,
                                int64_t b_cols, float* C) {
  for (int64_t i = r0; i < r1; i++)
    for (int64_t nz = rowptr[i]; nz < rowptr[i + 1]; nz++) {
      int64_t col = colidx[nz];
      float v = val[nz];
      for (int64_t j = 0; j < b_cols; j++) C[i + j * ld] += v * B[col + j * ld];
    }
}

}  // extern "C"
