// reorder.cpp — Jaccard row reordering (the Keeper algorithm), host side.
//
// Bit-exact with the reference's IterativeBlockingKeeper
// (preprocess/src/general/blocking.cpp:431-547, selected by
// `Matrix_Blocking -a 5`) followed by get_fixed_size_grouping and
// get_permutation (preprocess/src/general/utilities.cpp:8-20, 45-54).
//
// The seed loop is sequential by nature (a merge changes the group pattern
// that later candidates are measured against). This implementation keeps
// that order but evaluates candidate distances speculatively in parallel:
// a chunk of candidates is measured against the current pattern, then the
// chunk is committed in order up to the first merge, and measuring resumes
// after it with the grown pattern. Distances are computed on each row's
// sequence of block-column runs, which is exactly what the reference's
// distance walk consumes. The chunk is measured on the host's cores, or on a
// GPU (reorder_gpu.cu) with larger chunks; the commit is the same code
// either way, so both give the same grouping.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <numeric>
#include "keeper_set.h"
#include "smat_internal.h"

namespace smat {
namespace {

// Block ids of a column list with consecutive repeats collapsed
// (JaccardDistanceGroup skips runs of equal `col / block_size`).
void block_runs(const int64_t* c, int64_t n, int64_t bs, std::vector<int64_t>& out) {
  out.clear();
  for (int64_t i = 0; i < n; i++) {
    int64_t p = c[i] / bs;
    if (out.empty() || out.back() != p) out.push_back(p);
  }
}

// JaccardDistanceGroup (blocking.cpp:904-975) on run sequences, candidate
// group size 1.
inline float jaccard_runs(const int64_t* a, int64_t na, int64_t ga, const int64_t* b, int64_t nb) {
  if (na == 0 && nb == 0) return 0;
  if (na == 0 || nb == 0) return 1;
  int64_t i = 0, j = 0, count = 0, blocks_a = 0, blocks_b = 0;
  while (i < na && j < nb) {
    if (a[i] < b[j]) {
      count += 1; blocks_a++; i++;
    } else if (a[i] > b[j]) {
      count += ga; blocks_b++; j++;
    } else {
      blocks_a++; blocks_b++; i++; j++;
    }
  }
  blocks_a += na - i;
  count += na - i;
  blocks_b += nb - j;
  count += (nb - j) * ga;
  return (float)((2.0 * count) / (double)(blocks_a * ga + blocks_b + count));
}

// merge_rows (utilities.cpp:145-173), including its early exit that drops the
// tail of the pattern.
void merge_rows(std::vector<int64_t>& A, const int64_t* B, int64_t nb, std::vector<int64_t>& tmp) {
  tmp.clear();
  auto i = A.begin();
  int64_t j = 0;
  while (j < nb) {
    int64_t bv = B[j];
    auto ni = std::lower_bound(i, A.end(), bv);
    if (ni == A.end()) break;
    tmp.insert(tmp.end(), i, ni);
    tmp.push_back(bv);
    if (*ni == bv) ++ni;
    i = ni;
    j++;
  }
  tmp.insert(tmp.end(), B + j, B + nb);
  A.swap(tmp);
}

}  // namespace

bool keeper_grouping(int64_t rows, const int64_t* rowptr, const int32_t* cols32, float tau, int64_t bs,
                     int64_t max_b, std::vector<int64_t>& grouping, int64_t& comparisons, int64_t& merges,
                     KeeperDevice* dev) {
  const int64_t nnz = rowptr[rows];
  std::vector<int64_t> cols(cols32, cols32 + nnz);
  // per-row run sequences
  std::vector<int64_t> run_ptr(rows + 1, 0);
  std::vector<int64_t> runs;
  runs.reserve(nnz);
  {
    std::vector<int64_t> tmp;
    for (int64_t r = 0; r < rows; r++) {
      block_runs(cols.data() + rowptr[r], rowptr[r + 1] - rowptr[r], bs, tmp);
      runs.insert(runs.end(), tmp.begin(), tmp.end());
      run_ptr[r + 1] = (int64_t)runs.size();
    }
  }
  if (dev && !dev->init(runs, run_ptr)) return false;
  // chunk sizes: the device pays a round trip per chunk, so it measures every
  // remaining candidate at once (one launch per seed and per merge); on the
  // host a chunk starts at 1024 candidates (measured against 64 and 4096 on
  // an R-MAT 2^15 pattern: 4.9 s against 6.0 and 5.8 s on 8 threads)
  const int64_t chunk0 = dev ? std::max<int64_t>(rows, 1) : 1024;
  const int64_t chunk_max = dev ? std::max<int64_t>(rows, 1) : (int64_t)1 << 16;
  grouping.assign(rows, -1);
  // `float distances[rows] = {-1}` (GCC VLA initialiser): [-1, 0, 0, ...]
  std::vector<float> distances(rows, 0.0f);
  if (rows > 0) distances[0] = -1;
  std::vector<float> dbuf(rows);
  comparisons = 0;
  merges = 0;
  std::vector<int64_t> pattern, pruns, tmp;
  std::vector<int64_t> merged;
  KeeperBestSet best;  // the seed's best non-merged candidates (keeper_set.h)
  for (int64_t i = 0; i < rows; i++) {
    if (grouping[i] != -1) continue;
    best.clear();
    merged.clear();
    const int64_t gn = i + rows;
    pattern.assign(cols.begin() + rowptr[i], cols.begin() + rowptr[i + 1]);
    block_runs(pattern.data(), (int64_t)pattern.size(), bs, pruns);
    int64_t gsize = 1;
    grouping[i] = gn;
    merged.push_back(i);
    const float di = distances[i];
    int64_t j = i + 1;
    int64_t chunk = chunk0;
    while (j < rows && gsize != max_b) {
      const int64_t j1 = std::min<int64_t>(rows, j + chunk);
      const int64_t* pr = pruns.data();
      const int64_t npr = (int64_t)pruns.size();
      const int64_t g = gsize;
      if (dev) {
        if (!dev->fill(pr, npr, g, j, j1, dbuf.data() + j)) return false;
      } else {
#pragma omp parallel for schedule(dynamic, 256) if (j1 - j >= 256)
        for (int64_t jj = j; jj < j1; jj++) {
          const float dj = distances[jj];
          if (di != -1 && dj != -1 && std::fabs(di - dj) > tau) continue;
          if (grouping[jj] != -1) continue;
          dbuf[jj] = jaccard_runs(pr, npr, g, runs.data() + run_ptr[jj], run_ptr[jj + 1] - run_ptr[jj]);
        }
      }
      int64_t merged_at = -1;
      for (int64_t jj = j; jj < j1; jj++) {
        const float dj = distances[jj];
        if (di != -1 && dj != -1 && std::fabs(di - dj) > tau) {
          distances[jj] = -1;
          continue;
        }
        if (grouping[jj] != -1) continue;
        comparisons++;
        const float d = dbuf[jj];
        distances[jj] = d;
        if (d <= tau) {
          merges++;
          grouping[jj] = gn;
          merged.push_back(jj);
          merge_rows(pattern, cols.data() + rowptr[jj], rowptr[jj + 1] - rowptr[jj], tmp);
          block_runs(pattern.data(), (int64_t)pattern.size(), bs, pruns);
          gsize++;
          merged_at = jj;
          break;
        }
        // insert, then the reference's trim from end() (blocking.cpp:499-510)
        best.insert(d, jj);
        best.trim_from_end((size_t)max_b - merged.size());
      }
      if (merged_at >= 0) {
        j = merged_at + 1;
        chunk = chunk0;
      } else {
        j = j1;
        chunk = std::min<int64_t>(chunk * 4, chunk_max);
      }
    }
    if (gsize < max_b) {
      for (int32_t it = best.first(); it != KeeperBestSet::kEnd && gsize != max_b; it = best.next(it)) {
        grouping[best.row(it)] = gn;
        merged.push_back(best.row(it));
        gsize++;
      }
    }
    if (gsize == max_b)
      for (int64_t idx : merged) grouping[idx] -= rows;
  }
  return true;
}

std::vector<int64_t> permutation_of(const std::vector<int64_t>& grouping) {
  // utilities.cpp:8-20: unstable std::sort of iota by group id; the tie order
  // is libstdc++'s, which this file is built against as well.
  auto comp = [&](int i, int j) { return grouping[i] < grouping[j]; };
  std::vector<int64_t> v(grouping.size());
  std::iota(v.begin(), v.end(), 0);
  std::sort(v.begin(), v.end(), comp);
  return v;
}

std::vector<int64_t> fixed_size_grouping(const std::vector<int64_t>& grouping, int64_t row_block) {
  std::vector<int64_t> out(grouping.size(), -1);
  std::vector<int64_t> perm = permutation_of(grouping);
  for (int64_t i = 0; i < (int64_t)perm.size(); i++) out[perm[i]] = i / row_block;
  return out;
}

}  // namespace smat
