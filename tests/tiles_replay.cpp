// tiles_replay.cpp — TEST HARNESS: the merged-tile build of csrc/tiles.cu
// replayed on the CPU, step by step, with the same per-element functions
// (csrc/tiles_core.h) and plain loops in place of the kernels' threads and
// scans, so that the index arithmetic of the GPU build can be checked against
// the oracle without a GPU. Built into a shared library by
// tests/test_tiles_host.py.
#include <cstdint>
#include <cstring>
#include <vector>

#include "tiles_core.h"

using namespace smat::tiles;

extern "C" {

// Same outputs as the library's smat_tiles_copy_to_host, sized by a first
// call with out_rowptr == NULL (returns the tile count, sets *n_rowptr).
// Returns -1 - (fault flags) for rejected input, -100 if the labels built
// block by block differ from the labels read off the whole tiles.
int64_t replay_tiles(int64_t m_row, int64_t m_col, int k, int64_t nnzb, const int32_t* rowptr,
                     const int32_t* colidx, const uint16_t* vals, int64_t* n_rowptr, int32_t* out_rowptr,
                     int32_t* out_colidx, uint16_t* out_val, int32_t* out_info, int32_t* out_rel,
                     int32_t* out_labels) {
  const Geom g = make_geom(m_row, m_col, k, nnzb);
  int bad = 0;
  for (int64_t r = 0; r < g.nbr; ++r) bad |= check_row(g, rowptr, r);
  if (bad) return -1 - bad;
  std::vector<int32_t> maker(nnzb), is_maker(nnzb), tile_no(nnzb), brow(nnzb);
  for (int64_t i = 0; i < nnzb; ++i) {
    const int64_t r = block_row_of(rowptr, g.nbr, i);
    brow[i] = (int32_t)r;
    int b = 0;
    int64_t m = tile_maker(g, rowptr, colidx, i, r, &b);
    if (b) {
      bad |= b;
      m = i;
    }
    maker[i] = (int32_t)m;
    is_maker[i] = m == i;
  }
  if (bad) return -1 - bad;
  int32_t nt = 0;
  for (int64_t i = 0; i < nnzb; ++i) {
    tile_no[i] = nt;
    nt += is_maker[i];
  }
  std::vector<int32_t> tile_row(nt), tile_col(nt), start(nt), rank(nt);
  const int64_t cells = g.tile_rows * g.tile_cols;
  std::vector<int32_t> info(cells, 0), rel(cells);
  std::vector<uint16_t> tv((size_t)nt * g.tsz, 0);
  std::vector<int32_t> tile_of_block(nnzb);
  for (int64_t i = 0; i < nnzb; ++i) {
    const int64_t m = maker[i];
    const int32_t t = tile_no[m];
    tile_of_block[i] = t;
    if (m == i) {
      const int64_t x = colidx[i] / g.tw, y = brow[i] / 4;
      tile_col[t] = (int32_t)(x * g.tw);
      tile_row[t] = (int32_t)y;
      info[y * g.tile_cols + x] = 1;
    }
  }
  std::vector<int32_t> flags((size_t)nt * 16, 0);
  for (int64_t i = 0; i < nnzb; ++i) {
    const int64_t r = brow[i];
    const int64_t off = (int64_t)tile_of_block[i] * g.tsz + block_offset_in_tile(g, r, colidx[i]);
    std::memcpy(tv.data() + off, vals + i * 16 * k, sizeof(uint16_t) * 16 * k);
    int f[4];
    block_label_flags(g, vals + i * 16 * k, f);
    for (int sc = 0; sc < 4; ++sc) flags[(size_t)tile_of_block[i] * 16 + 4 * (r % 4) + sc] |= f[sc];
  }
  // the block-wise flags must give the labels the reference reads off the whole tile
  for (int64_t e = 0; e < (int64_t)nt * 16; ++e)
    if (label_of_flags(flags[e]) != tile_label(g, tv.data() + (e / 16) * g.tsz, (int)(e % 16))) return -100;
  int32_t used = 0;
  for (int64_t t = 0; t < nt; ++t) {
    start[t] = (t == 0 || tile_row[t - 1] != tile_row[t]);
    rank[t] = used;
    used += start[t];
  }
  std::vector<int32_t> rp(used + 1, 0);
  for (int64_t t = 0; t < nt; ++t)
    if (start[t]) rp[rank[t]] = (int32_t)t;
  rp[used] = nt;
  int32_t run = 0;
  for (int64_t c = 0; c < cells; ++c) {
    rel[c] = info[c] ? run : -1;
    run += info[c];
  }
  if (n_rowptr) *n_rowptr = used + 1;
  if (!out_rowptr) return nt;
  std::memcpy(out_rowptr, rp.data(), sizeof(int32_t) * rp.size());
  std::memcpy(out_colidx, tile_col.data(), sizeof(int32_t) * nt);
  std::memcpy(out_val, tv.data(), sizeof(uint16_t) * tv.size());
  std::memcpy(out_info, info.data(), sizeof(int32_t) * cells);
  std::memcpy(out_rel, rel.data(), sizeof(int32_t) * cells);
  for (int64_t e = 0; e < (int64_t)nt * 16; ++e) out_labels[e] = label_of_flags(flags[e]);
  return nt;
}
}
