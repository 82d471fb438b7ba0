// sp24.cpp — host side of the structured-sparse (2:4) path: the units,
// stages and groups of spmm24.h, and the compressed stream.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "fp_convert.h"
#include "smat_internal.h"
#include "spmm24.h"

namespace smat {

namespace {

// Kept values and metadata nibble of one group of four 16-bit values whose
// nonzeros (judged on the FP16 bits) are at most two: the two kept
// positions i0 < i1 (nonzero positions first, then the lowest free ones),
// nibble = i0 | i1 << 2.
inline uint32_t compress_group(const uint16_t* f16, const uint16_t* out_vals, uint16_t kept[2]) {
  int pos[2], n = 0;
  for (int i = 0; i < 4 && n < 2; i++)
    if ((f16[i] & 0x7fffu) != 0) pos[n++] = i;
  if (n == 0) {
    pos[0] = 0;
    pos[1] = 1;
  } else if (n == 1) {
    pos[1] = pos[0] < 3 ? pos[0] + 1 : 3;
    if (pos[0] == 3) pos[0] = 2;
  }
  // positions without a nonzero keep a zero value
  for (int q = 0; q < 2; q++) kept[q] = (f16[pos[q]] & 0x7fffu) != 0 ? out_vals[pos[q]] : 0;
  return (uint32_t)pos[0] | ((uint32_t)pos[1] << 2);
}

}  // namespace

void route_sp24(const HostBcsr& b, int min_unit, std::vector<uint8_t>& take) {
  const int64_t nbr = b.nbr(), nnzb = b.nnzb();
  take.assign(nnzb, 0);
  if (b.bh != 16 || b.bw != 16 || min_unit < 1) return;
  // count the exact-2:4 blocks of every unit of a group, window by window
  std::vector<int32_t> cnt;
  for (int64_t g0 = 0; g0 < nbr; g0 += kSp24GroupRows) {
    const int64_t g1 = std::min<int64_t>(nbr, g0 + kSp24GroupRows);
    for (int pass = 0; pass < 3; pass++)
      for (int64_t br = g0; br < g1; br++)
        for (int32_t k = b.rowptr[br]; k < b.rowptr[br + 1]; k++) {
          if (!b.is24[k]) continue;
          const int32_t w = b.colidx[k] / 32;
          if (pass == 0) {
            if ((size_t)w >= cnt.size()) cnt.resize((size_t)w + 1, 0);
            cnt[w]++;
          } else if (pass == 1) {
            take[k] = cnt[w] >= min_unit ? 1 : 0;
          } else {
            cnt[w] = 0;  // reset for the next group
          }
        }
  }
}

smat_status build_sp24(const HostBcsr& b, const std::vector<uint8_t>& take, int fmt, Sp24Host& out) {
  out = Sp24Host{};
  if (b.bh != 16 || b.bw != 16) return fail(SMAT_ERR_UNSUPPORTED, "2:4 path: 16 x 16 blocks only");
  const int64_t nbr = b.nbr();
  const int64_t ngroups = (nbr + kSp24GroupRows - 1) / kSp24GroupRows;
  struct Ent {
    int32_t window, bit;
    int64_t k;
  };
  std::vector<Ent> ent;
  std::vector<uint16_t> conv(256);
  for (int64_t g = 0; g < ngroups; g++) {
    ent.clear();
    uint32_t row_mask = 0;
    for (int j = 0; j < kSp24GroupRows; j++) {
      const int64_t br = g * kSp24GroupRows + j;
      if (br >= nbr) break;
      for (int32_t k = b.rowptr[br]; k < b.rowptr[br + 1]; k++)
        if (take[k]) {
          const int32_t kb = b.colidx[k] / 16;
          ent.push_back({kb / 2, 2 * j + (kb & 1), k});
          row_mask |= 1u << j;
        }
    }
    if (ent.empty()) continue;
    std::sort(ent.begin(), ent.end(),
              [](const Ent& x, const Ent& y) { return x.window != y.window ? x.window < y.window : x.bit < y.bit; });
    Sp24Group G{};
    G.group = (int32_t)g;
    G.row_mask = row_mask;
    G.stage0 = (int32_t)out.stages.size();
    G.unit0 = (int32_t)out.unit_window.size();
    // units, then stages of whole units
    size_t e = 0;
    std::vector<std::pair<size_t, size_t>> units;  // [first, last) entries
    while (e < ent.size()) {
      size_t f = e;
      while (f < ent.size() && ent[f].window == ent[e].window) f++;
      units.push_back({e, f});
      e = f;
    }
    size_t u = 0;
    while (u < units.size()) {
      size_t v = u;
      int nblk = 0;
      while (v < units.size() && (int)(v - u) < kSp24StageUnits &&
             nblk + (int)(units[v].second - units[v].first) <= kSp24StageBlocks) {
        nblk += (int)(units[v].second - units[v].first);
        v++;
      }
      const int nu = (int)(v - u);
      Sp24Stage S{};
      S.off = (int64_t)out.stream.size();
      S.nunits = nu;
      S.nblk = nblk;
      S.unit0 = (int32_t)(out.unit_window.size() - (size_t)G.unit0);
      S.bytes = nu * (int32_t)sizeof(Sp24Unit) + nblk * kSp24BlockBytes;
      out.stream.resize(out.stream.size() + (size_t)S.bytes, 0);
      uint8_t* base = out.stream.data() + S.off;
      uint8_t* vals = base + (size_t)nu * sizeof(Sp24Unit);
      uint8_t* metas = vals + (size_t)nblk * 256;
      int bi = 0;
      for (size_t x = u; x < v; x++) {
        Sp24Unit U{};
        U.window = ent[units[x].first].window;
        U.first = (uint16_t)bi;
        for (size_t y = units[x].first; y < units[x].second; y++, bi++) {
          const Ent& en = ent[y];
          U.mask = (uint16_t)(U.mask | (1u << en.bit));
          const uint16_t* f16 = b.val_f16.data() + (size_t)en.k * 256;
          const uint16_t* src = f16;
          if (fmt == 1) {
            for (int i = 0; i < 256; i++) conv[i] = f32_to_bf16_bits(b.val[(size_t)en.k * 256 + i]);
            src = conv.data();
          }
          for (int rr = 0; rr < 16; rr++) {
            uint16_t kept[8];
            uint32_t m16 = 0;
            for (int q = 0; q < 4; q++)
              m16 |= compress_group(f16 + rr * 16 + 4 * q, src + rr * 16 + 4 * q, kept + 2 * q) << (4 * q);
            std::memcpy(vals + (size_t)bi * 256 + rr * 16, kept, 16);
            const uint16_t m = (uint16_t)m16;
            std::memcpy(metas + (size_t)bi * 32 + rr * 2, &m, 2);
          }
        }
        std::memcpy(base + (x - u) * sizeof(Sp24Unit), &U, sizeof(U));
        out.unit_window.push_back(U.window);
      }
      out.stages.push_back(S);
      out.n_blocks += nblk;
      u = v;
    }
    G.nstages = (int32_t)out.stages.size() - G.stage0;
    G.nunits = (int32_t)out.unit_window.size() - G.unit0;
    out.groups.push_back(G);
  }
  out.n_units = (int64_t)out.unit_window.size();
  // heaviest groups first: the CTAs take them round-robin
  std::stable_sort(out.groups.begin(), out.groups.end(),
                   [](const Sp24Group& x, const Sp24Group& y) { return x.nunits > y.nunits; });
  if (out.stream.empty()) out.stream.resize(16, 0);
  return SMAT_OK;
}

}  // namespace smat
