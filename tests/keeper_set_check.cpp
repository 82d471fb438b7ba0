// Checks KeeperBestSet (sptc-smat_gb300/csrc/keeper_set.h) against the
// container the reference scan uses, std::set<std::pair<float, long>>, under
// the reference's operations (preprocess/src/general/blocking.cpp:499-510 and
// 517-523): insert a (distance, row) key, then, when the set holds more than
// `keep` keys, advance an iterator `keep` steps from end() and erase from there
// to end(); at the end of a seed, walk the keys in order. Random sequences
// with many equal distances and keep values from 1 to 16; the two sets must
// hold the same keys in the same order after every operation.
#include <cstdint>
#include <cstdio>
#include <iterator>
#include <random>
#include <set>
#include <utility>

#include "keeper_set.h"

int main() {
  std::mt19937_64 rng(12345);
  long checks = 0, bad = 0;
  for (int seq = 0; seq < 2000 && bad == 0; seq++) {
    std::set<std::pair<float, long>> ref;
    smat::KeeperBestSet mine;
    const int ops = 50 + (int)(rng() % 3000);
    const int levels = 1 + (int)(rng() % 40);   // few distinct distances: many ties
    const size_t keep_base = 1 + rng() % 16;
    size_t keep = keep_base;
    for (int op = 0; op < ops; op++) {
      const float d = (float)(rng() % levels) / (float)levels;
      const long j = op;
      if (rng() % 97 == 0 && keep > 1) keep--;  // a merge lowers keep
      ref.insert({d, j});
      mine.insert(d, j);
      if (ref.size() > keep) {
        auto it = ref.end();
        std::advance(it, keep);
        ref.erase(it, ref.end());
      }
      mine.trim_from_end(keep);
      checks++;
      if (ref.size() != mine.size()) {
        bad++;
        std::printf("seq %d op %d: size %zu vs %zu\n", seq, op, ref.size(), mine.size());
        break;
      }
      int32_t x = mine.first();
      for (const auto& kv : ref) {
        if (x == smat::KeeperBestSet::kEnd || mine.dist(x) != kv.first || mine.row(x) != kv.second) {
          bad++;
          std::printf("seq %d op %d: contents differ\n", seq, op);
          break;
        }
        x = mine.next(x);
      }
      if (bad) break;
      if (x != smat::KeeperBestSet::kEnd) {
        bad++;
        std::printf("seq %d op %d: extra keys\n", seq, op);
        break;
      }
      if (rng() % 500 == 0) {  // a new seed starts with an empty set
        ref.clear();
        mine.clear();
        keep = keep_base;
      }
    }
  }
  std::printf("%ld states compared, %ld mismatches\n", checks, bad);
  if (bad == 0) std::printf("ALL OK\n");
  return bad == 0 ? 0 : 1;
}
