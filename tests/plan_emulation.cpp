// CPU replay of the tensor-core kernel's use of a work plan (test driver).
//
// Builds the plan the library builds (csrc/bcsr.cpp: build_host_bcsr,
// build_plan, build_work_items) for seeded matrices and replays, in FP64,
// what the kernel does with it:
//   * every stage's MMA entries (tile, position, slot, run length,
//     accumulate flag) against the stage's block list and B tiles;
//   * per TMEM slot, overwrite on the first block and accumulate after it;
//   * the epilogue: a hub row's later parts (ext_mask) added into its first
//     part, C rows through the plan's row map;
//   * split panels: each part on zeroed accumulators, parts summed.
// Checks the plan's invariants on the way and compares C with an FP64 CSR
// product. Prints one line per case and "ALL OK" or "FAIL"; exit status 0
// on success.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "smat_internal.h"

namespace smat {
void set_error(const std::string& m) { std::fprintf(stderr, "error: %s\n", m.c_str()); }
smat_status fail(smat_status st, const std::string& m) {
  set_error(m);
  return st;
}
}  // namespace smat

using namespace smat;

namespace {

enum Shape { kRandom, kClustered, kHubs };

struct Case {
  int64_t rows, cols;
  double dens;
  Shape shape;
  unsigned seed;
};

int check(bool ok, const char* what) {
  if (!ok) std::printf("  violated: %s\n", what);
  return ok ? 0 : 1;
}

// C contribution of one block (bh x 16) times the B rows of its block column.
void add_block(const HostBcsr& hb, int32_t blk, int kb, const std::vector<double>& B, int N, double* dst,
               bool overwrite) {
  const int bh = hb.bh;
  for (int i = 0; i < bh; i++)
    for (int n = 0; n < N; n++) {
      double s = 0;
      for (int j = 0; j < 16; j++) s += (double)hb.val[(size_t)blk * bh * 16 + i * 16 + j] * B[(size_t)(kb * 16 + j) * N + n];
      double& d = dst[(size_t)i * N + n];
      d = overwrite ? s : d + s;
    }
}

// Replays stages [s0, s1) of panel p onto acc (R slots x bh rows x N);
// returns the number of invariant violations.
int replay(const HostBcsr& hb, const Plan& pl, int R, int cls, int p, int s0, int s1, const std::vector<double>& B,
           int N, std::vector<double>& acc, std::vector<int>& seen) {
  const int bh = hb.bh;
  const PanelInfo& pi = pl.panels[p];
  const int PW = R % kMmaWarps == 0 ? R / kMmaWarps : 0;
  int bad = 0;
  for (int c = s0; c < s1; c++) {
    const StageRec& st = pl.stages[pi.stage_off + c];
    bad += check(st.nblk >= 1 && st.nblk <= stage_rows(cls) / bh, "blocks per stage");
    bad += check(st.ntiles >= 1 && st.ntiles <= stage_tiles(cls), "tiles per stage");
    const uint8_t* h = pl.headers.data() + st.hdr_off;
    uint16_t wl[kMmaWarps];
    std::memcpy(wl, h, sizeof(wl));
    int covered = 0;
    for (int w = 0; w < kMmaWarps; w++) {
      for (int e = 0; e < (wl[w] >> 8); e++) {
        uint32_t m;
        std::memcpy(&m, h + kStageHdrFixed + 4 * ((wl[w] & 0xff) + e), 4);
        const int pos = m & 31, tile = (m >> 5) & 15, slot = (m >> 9) & 31, len = ((m >> 14) & 15) + 1;
        const bool accumulate = (m >> 18) & 1;
        bad += check(tile < st.ntiles && pos + len <= st.nblk && slot + len <= R, "entry in range");
        bad += check((uint32_t)((slot * kMmaWarps) / R) == (uint32_t)w &&
                         (uint32_t)(((slot + len - 1) * kMmaWarps) / R) == (uint32_t)w,
                     "slots owned by the issuing warp");
        for (int q = 0; q < len; q++) {
          const int32_t blk = pl.stream_blk[st.blk_off + pos + q];
          const int sl = slot + q;
          seen[blk]++;
          covered++;
          // the slot's block row: its own row-map entry, or its chain head's
          int head = sl;
          while (PW && ((pi.ext_mask >> head) & 1u)) head -= PW;
          const int32_t row0 = pl.row_map[((size_t)p * R + head) * bh];
          bad += check(row0 >= 0, "slot with blocks has C rows");
          if (row0 < 0) continue;
          const int64_t br = row0 / bh;
          bad += check(hb.rowptr[br] <= blk && blk < hb.rowptr[br + 1], "block belongs to the slot's row");
          bad += check(hb.colidx[blk] / 16 == st.kb[tile], "tile is the block's column");
          add_block(hb, blk, st.kb[tile], B, N, &acc[(size_t)sl * bh * N], !accumulate);
        }
      }
    }
    bad += check(covered == st.nblk, "every block of the stage in one MMA entry");
  }
  return bad;
}

// Epilogue: chain parts added into their head, written to C by row map.
void epilogue(const Plan& pl, int R, int bh, int p, const std::vector<double>& acc, int N, std::vector<double>& C) {
  const PanelInfo& pi = pl.panels[p];
  const int PW = R % kMmaWarps == 0 ? R / kMmaWarps : 0;
  for (int s = 0; s < R; s++) {
    if ((pi.ext_mask >> s) & 1u) continue;
    for (int i = 0; i < bh; i++) {
      const int32_t row = pl.row_map[((size_t)p * R + s) * bh + i];
      if (row < 0) continue;
      for (int n = 0; n < N; n++) {
        double v = acc[((size_t)s * bh + i) * N + n];
        if (PW)
          for (int t = s + PW; t < R && ((pi.ext_mask >> t) & 1u); t += PW) v += acc[((size_t)t * bh + i) * N + n];
        C[(size_t)row * N + n] += v;
      }
    }
  }
}

double rel_err(const std::vector<double>& a, const std::vector<double>& b) {
  double e = 0, n = 0;
  for (size_t i = 0; i < a.size(); i++) {
    e += (a[i] - b[i]) * (a[i] - b[i]);
    n += b[i] * b[i];
  }
  return std::sqrt(e / std::max(n, 1e-300));
}

int run(const Case& cs, int bh, int R, int cls) {
  std::mt19937_64 rng(cs.seed);
  std::uniform_real_distribution<double> U(0, 1);
  std::vector<int64_t> rp(cs.rows + 1, 0);
  std::vector<int32_t> ci;
  std::vector<float> v;
  for (int64_t r = 0; r < cs.rows; r++) {
    for (int64_t c = 0; c < cs.cols; c++) {
      double d = cs.dens;
      if (cs.shape == kClustered) d = ((c / 16) % 7 == (r / 16) % 7) ? 0.3 : cs.dens * 0.2;
      if (cs.shape == kHubs) d = (r % 97 == 5 || r % 211 == 17) ? 0.6 : cs.dens;
      if (U(rng) < d) {
        ci.push_back((int32_t)c);
        v.push_back((float)(U(rng) * 2 - 1));
      }
    }
    rp[r + 1] = (int64_t)ci.size();
  }
  smat_csr A{cs.rows, cs.cols, (int64_t)ci.size(), rp.data(), ci.data(), v.data(), 0};
  HostBcsr hb;
  Plan pl;
  if (build_host_bcsr(A, bh, 16, nullptr, hb) != SMAT_OK || build_plan(hb, R, cls, pl) != SMAT_OK) return 1;
  const int N = 4;
  std::vector<double> B((size_t)hb.cols_p * N);
  for (auto& x : B) x = U(rng) * 2 - 1;
  std::vector<double> Cref((size_t)hb.rows_p * N, 0.0);
  for (int64_t r = 0; r < cs.rows; r++)
    for (int64_t k = rp[r]; k < rp[r + 1]; k++)
      for (int n = 0; n < N; n++) Cref[r * N + n] += (double)v[k] * B[(size_t)ci[k] * N + n];
  int bad = 0;
  // whole panels
  {
    std::vector<double> C(Cref.size(), 0.0);
    std::vector<int> seen(hb.nnzb(), 0);
    for (int p = 0; p < pl.n_panels; p++) {
      std::vector<double> acc((size_t)R * bh * N, 0.0);
      bad += replay(hb, pl, R, cls, p, 0, pl.panels[p].nstages, B, N, acc, seen);
      epilogue(pl, R, bh, p, acc, N, C);
    }
    for (int64_t k = 0; k < hb.nnzb(); k++) bad += check(seen[k] == 1, "every block exactly once");
    const double e = rel_err(C, Cref);
    bad += check(e < 1e-12, "whole-panel result vs FP64");
    std::printf("rows %ld cols %ld bh %d R %d class %d: panels %d stages %zu blocks %ld err %.2g\n", (long)cs.rows,
                (long)cs.cols, bh, R, cls, pl.n_panels, pl.stages.size(), (long)hb.nnzb(), e);
  }
  // split parts: few workers and a small threshold force splits
  {
    std::vector<WorkItem> items;
    std::vector<int32_t> order;
    int32_t n_split = 0, n_slabs = 0;
    build_work_items(pl, bh, 7, 0.05, items, order, n_split, n_slabs);
    std::vector<int> taken(items.size(), 0);
    for (int32_t i : order) taken[i]++;
    for (int t : taken) bad += check(t == 1, "order lists every item once");
    std::vector<double> C(Cref.size(), 0.0);
    std::vector<int> seen(hb.nnzb(), 0), stage_done(pl.stages.size(), 0);
    for (const WorkItem& w : items) {
      const PanelInfo& pi = pl.panels[w.panel];
      bad += check(w.s0 >= 0 && w.s0 < w.s1 && w.s1 <= pi.nstages, "item stage range");
      bad += check(w.split >= 0 || (w.s0 == 0 && w.s1 == pi.nstages), "an unsplit item is the whole panel");
      bad += check(w.split < 0 || (w.nparts >= 2 && w.nparts <= pi.nstages / 4), "at most one part per four stages");
      for (int c = w.s0; c < w.s1; c++) stage_done[pi.stage_off + c]++;
      std::vector<double> acc((size_t)R * bh * N, 0.0);  // a part starts on zeroed accumulators
      bad += replay(hb, pl, R, cls, w.panel, w.s0, w.s1, B, N, acc, seen);
      epilogue(pl, R, bh, w.panel, acc, N, C);
    }
    for (int d : stage_done) bad += check(d == 1, "every stage in one item");
    const double e = rel_err(C, Cref);
    bad += check(e < 1e-12, "split-part result vs FP64");
    std::printf("  items %zu split panels %d slabs %d err %.2g\n", items.size(), n_split, n_slabs, e);
  }
  return bad;
}

}  // namespace

int main() {
  const Case cases[] = {{1000, 997, 0.05, kRandom, 1},
                        {700, 1300, 0.02, kClustered, 7},
                        {513, 260, 0.4, kRandom, 3},
                        {2000, 3000, 0.004, kHubs, 11}};
  int bad = 0;
  for (const Case& cs : cases)
    for (int bh : {16, 32})
      for (int R : {4, 8, 16}) {
        if (bh == 32 && R > 8) continue;
        for (int cls = 0; cls < kPlanClasses; cls++) {
          if (cls == 2 && bh != 16) continue;  // FP8 form: 16-row blocks only
          bad += run(cs, bh, R, cls);
        }
      }
  std::printf(bad ? "FAIL\n" : "ALL OK\n");
  return bad ? 1 : 0;
}
