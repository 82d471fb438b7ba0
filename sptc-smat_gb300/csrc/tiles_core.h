// tiles_core.h — per-element steps of the merged-tile build (tiles.cu).
//
// The reference's SparseMatrix::bcsrBlocking (src/cuda_hgemm/src/common/
// matrix.h:794-1137) groups the 16 x k blocks of a BCSR into TILES of 4 x 4
// blocks (64 rows x 4k columns) with one sequential pass that searches the
// tiles made so far for every block (quadratic in the block count). Its
// result is fixed by three facts, which make every step here independent per
// element:
//   * a tile is made by the FIRST block, in BCSR order, that falls into it;
//     within its tile row that is the earliest block row holding a block of
//     the tile's column range, at the lowest index there (block columns are
//     ascending inside a block row), so each block finds its tile's maker by
//     at most three binary searches in the block rows above it;
//   * tiles are numbered in the order their makers appear, so a tile's number
//     is the count of makers before its own (an exclusive scan of the
//     "maker" flags);
//   * the tile row pointer holds one entry per tile row that has a tile (the
//     reference skips empty tile rows), so its entries are the numbers of the
//     tiles that start a tile row, ranked by another scan.
// The functions are __host__ __device__ so that a CPU replay of the same
// arithmetic can check it against the reference (tests/tiles_replay.cpp).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define SMAT_TILES_HD __host__ __device__ __forceinline__
#else
#define SMAT_TILES_HD inline
#endif

namespace smat {
namespace tiles {

// Shape of one build: BCSR of m_row x m_col in 16 x k blocks (m_row a
// multiple of 16, m_col of k), tiles of 64 x 4k.
struct Geom {
  int64_t m_row, m_col, nnzb;
  int32_t k;
  int64_t nbr;       // block rows, m_row / 16
  int64_t tw;        // tile width in columns, 4k
  int64_t tile_rows; // ceil(m_row / 64)
  int64_t tile_cols; // ceil(m_col / 4k)
  int64_t tsz;       // values per tile, 256k
};

inline Geom make_geom(int64_t m_row, int64_t m_col, int32_t k, int64_t nnzb) {
  Geom g;
  g.m_row = m_row;
  g.m_col = m_col;
  g.nnzb = nnzb;
  g.k = k;
  g.nbr = m_row / 16;
  g.tw = 4 * (int64_t)k;
  g.tile_rows = (m_row + 63) / 64;
  g.tile_cols = (m_col + g.tw - 1) / g.tw;
  g.tsz = 256 * (int64_t)k;
  return g;
}

// Input faults found by the checks below (bit flags).
enum : int { BAD_ROWPTR = 1, BAD_COLIDX = 2, BAD_ORDER = 4 };

// First index in [lo, hi) whose column start is >= v (colidx ascending there).
SMAT_TILES_HD int64_t lower_bound_col(const int32_t* colidx, int64_t lo, int64_t hi, int64_t v) {
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if ((int64_t)colidx[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// Block row of block i: the smallest r with rowptr[r + 1] > i, the row the
// reference's scan settles on (matrix.h:822-825). rowptr[nbr] > i.
SMAT_TILES_HD int64_t block_row_of(const int32_t* rowptr, int64_t nbr, int64_t i) {
  int64_t lo = 0, hi = nbr - 1;
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if ((int64_t)rowptr[mid + 1] > i)
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

// Check of block row r's pointer pair (r in [0, nbr)); the pointer array
// must start at 0, never decrease and end at nnzb.
SMAT_TILES_HD int check_row(const Geom& g, const int32_t* rowptr, int64_t r) {
  int bad = 0;
  if (rowptr[r] > rowptr[r + 1]) bad |= BAD_ROWPTR;
  if (r == 0 && rowptr[0] != 0) bad |= BAD_ROWPTR;
  if (r == g.nbr - 1 && (int64_t)rowptr[g.nbr] != g.nnzb) bad |= BAD_ROWPTR;
  return bad;
}

// Step 1, block i in block row r (row pointers already checked): the index
// of the block that made i's tile (i itself when i makes it), or -1 with
// *bad set when i's column start is out of range, not a multiple of k, or
// not above the previous block's in the same block row.
SMAT_TILES_HD int64_t tile_maker(const Geom& g, const int32_t* rowptr, const int32_t* colidx, int64_t i, int64_t r,
                                 int* bad) {
  const int64_t col = colidx[i];
  if (col < 0 || col >= g.m_col || col % g.k != 0) {
    *bad |= BAD_COLIDX;
    return -1;
  }
  if (i > (int64_t)rowptr[r] && (int64_t)colidx[i - 1] >= col) {
    *bad |= BAD_ORDER;
    return -1;
  }
  const int64_t x0 = col - col % g.tw, x1 = x0 + g.tw;
  for (int64_t b = r - r % 4; b < r; ++b) {
    const int64_t j = lower_bound_col(colidx, rowptr[b], rowptr[b + 1], x0);
    if (j < (int64_t)rowptr[b + 1] && (int64_t)colidx[j] < x1) return j;
  }
  return lower_bound_col(colidx, rowptr[r], i + 1, x0);
}

// Step 2 places block i into tile t: offset of its first value inside the
// tile's values. Blocks sit block-major, k * 4 * (row offset) + 16 *
// (column offset) (matrix.h:851, :878-879).
SMAT_TILES_HD int64_t block_offset_in_tile(const Geom& g, int64_t r, int64_t col) {
  const int64_t by = r % 4, bx = (col % g.tw) / g.k;
  return 16 * (int64_t)g.k * (4 * by + bx);
}

// Labels. The reference labels position s (0..15) of a tile by reading the
// tile's values as a ROW-MAJOR 64 x 4k matrix, rows 16 (s / 4) .. +15,
// columns k (s % 4) .. +k-1 (matrix.h:1036-1088): 0 all zero, 1 no group of
// four with more than two nonzeros, 2 otherwise (a value is nonzero unless
// it is +0 or -0). The tile stores its blocks block-major, so row R of that
// view is the 4k values of rows 4 (R % 4) .. +3 of block R / 4, and columns
// k (s % 4) .. +k-1 of it are row 4 (R % 4) + s % 4 of that block: position
// (sr, sc) looks at the rows rho with rho % 4 == sc of the four blocks of the
// tile's block row sr. So each block can add its share while it is copied:
// flags per sc (bit 0: a nonzero, bit 1: a group of four with more than two),
// ORed into the position and turned into the label at the end.

// Flags of one group of four FP16 values given as two 32-bit words.
SMAT_TILES_HD int group_flags(uint32_t lo, uint32_t hi) {
  const int nz = ((lo & 0x7fffu) != 0) + ((lo & 0x7fff0000u) != 0) + ((hi & 0x7fffu) != 0) +
                 ((hi & 0x7fff0000u) != 0);
  return (nz > 0 ? 1 : 0) | (nz > 2 ? 2 : 0);
}

// Flags a block (16 x k values, row-major) adds to positions (by, 0..3) of
// its tile: flags[sc] from its rows rho with rho % 4 == sc.
SMAT_TILES_HD void block_label_flags(const Geom& g, const uint16_t* blk, int flags[4]) {
  for (int sc = 0; sc < 4; ++sc) flags[sc] = 0;
  for (int rho = 0; rho < 16; ++rho)
    for (int c = 0; c < g.k; c += 4) {
      const uint16_t* q = blk + rho * g.k + c;
      flags[rho % 4] |= group_flags((uint32_t)q[0] | ((uint32_t)q[1] << 16), (uint32_t)q[2] | ((uint32_t)q[3] << 16));
    }
}

// Label from the ORed flags of a position.
SMAT_TILES_HD int32_t label_of_flags(int v) { return (v & 2) ? 2 : (v & 1); }

// The label of position s read directly from a whole tile, as the reference
// reads it (the CPU replay checks the block-wise flags against it).
SMAT_TILES_HD int32_t tile_label(const Geom& g, const uint16_t* tile, int s) {
  const int sr = s / 4, sc = s % 4;
  bool any = false, two_four = true;
  for (int rr = 0; rr < 16; ++rr) {
    const uint16_t* row = tile + (int64_t)(16 * sr + rr) * g.tw + (int64_t)sc * g.k;
    for (int grp = 0; grp < g.k / 4; ++grp) {
      int nz = 0;
      for (int c = 0; c < 4; ++c) nz += (row[4 * grp + c] & 0x7fff) != 0;
      any = any || nz > 0;
      two_four = two_four && nz <= 2;
    }
  }
  return any ? (two_four ? 1 : 2) : 0;
}

}  // namespace tiles
}  // namespace smat
