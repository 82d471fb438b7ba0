// keeper_set.h — the Keeper scan's ordered set of best candidates.
//
// The reference keeps the best non-merged candidates of a seed in a
// std::set<std::pair<float, long>> and trims it after every insert by
// advancing an iterator from end() (preprocess/src/general/blocking.cpp:499-510).
// Advancing past end() of that red-black tree first steps to the smallest
// node of the subtree under the largest key and then walks in order, round
// through end() again, so which keys a trim removes depends on the tree's
// shape, not only on the keys. This set is a red-black tree with the same
// shape as the reference's container for the same operations: insertion and
// deletion follow the textbook algorithm (Cormen, Leiserson, Rivest, Stein,
// "Introduction to Algorithms", 3rd ed., ch. 13: RB-INSERT-FIXUP, RB-DELETE
// with RB-TRANSPLANT of the successor, RB-DELETE-FIXUP), which is the
// algorithm that container implements. Nodes live in one pooled array
// (indices, no allocation per key). tests/keeper_set_check.cpp checks it
// against std::set, operation by operation.
#pragma once

#include <cstdint>
#include <vector>

namespace smat {

class KeeperBestSet {
 public:
  static constexpr int32_t kNil = -1;
  static constexpr int32_t kEnd = -2;  // the position after the largest key

  void clear() {
    nodes_.clear();
    free_.clear();
    root_ = kNil;
    size_ = 0;
  }
  size_t size() const { return size_; }
  float dist(int32_t x) const { return nodes_[x].d; }
  int64_t row(int32_t x) const { return nodes_[x].j; }

  // Inserts a key that is not present (rows are unique).
  void insert(float d, int64_t j) {
    int32_t y = kNil, x = root_;
    bool left = false;
    while (x != kNil) {
      y = x;
      left = less(d, j, nodes_[x]);
      x = left ? nodes_[x].l : nodes_[x].r;
    }
    const int32_t z = alloc(d, j);
    nodes_[z].p = y;
    if (y == kNil)
      root_ = z;
    else if (left)
      nodes_[y].l = z;
    else
      nodes_[y].r = z;
    insert_fixup(z);
    size_++;
  }

  int32_t first() const { return root_ == kNil ? kEnd : leftmost(root_); }

  // In-order successor; kEnd after the largest key.
  int32_t next(int32_t x) const {
    if (nodes_[x].r != kNil) return leftmost(nodes_[x].r);
    int32_t y = nodes_[x].p;
    while (y != kNil && x == nodes_[y].r) {
      x = y;
      y = nodes_[y].p;
    }
    return y == kNil ? kEnd : y;
  }

  // The reference's trim, applied when the set holds more than `keep` keys:
  // it = end(); advance it by `keep`; erase [it, end()). From end() the
  // iterator steps to the smallest key under the largest one, walks in order
  // to the largest, then to end(), and round again: a cycle through the
  // largest key's subtree and end(). The largest key has no right child, so
  // its subtree holds at most 2 keys in a red-black tree, and the position
  // after `keep` steps is read off the cycle instead of walking it.
  void trim_from_end(size_t keep) {
    if (root_ == kNil || size_ <= keep) return;
    const int32_t mx = rightmost(root_);
    int32_t cyc[64];
    int n = 0;
    for (int32_t x = leftmost(mx);; x = next(x)) {
      cyc[n++] = x;
      if (x == mx || n == 64) break;
    }
    const size_t r = (keep - 1) % (size_t)(n + 1);  // keep >= 1 here (size > keep)
    int32_t it = r < (size_t)n ? cyc[r] : kEnd;
    if (it == kEnd) return;
    if (it == first()) {
      clear();
      return;
    }
    while (it != kEnd) {
      const int32_t nx = next(it);
      erase(it);
      it = nx;
    }
  }

 private:
  struct Node {
    float d;
    int64_t j;
    int32_t l, r, p;
    bool red;
  };

  static bool less(float d, int64_t j, const Node& b) { return d < b.d || (!(b.d < d) && j < b.j); }

  int32_t alloc(float d, int64_t j) {
    int32_t i;
    if (!free_.empty()) {
      i = free_.back();
      free_.pop_back();
    } else {
      i = (int32_t)nodes_.size();
      nodes_.push_back(Node{});
    }
    nodes_[i] = Node{d, j, kNil, kNil, kNil, true};
    return i;
  }

  int32_t leftmost(int32_t x) const {
    while (nodes_[x].l != kNil) x = nodes_[x].l;
    return x;
  }
  int32_t rightmost(int32_t x) const {
    while (nodes_[x].r != kNil) x = nodes_[x].r;
    return x;
  }
  bool red(int32_t x) const { return x != kNil && nodes_[x].red; }

  void rotate_left(int32_t x) {
    const int32_t y = nodes_[x].r;
    nodes_[x].r = nodes_[y].l;
    if (nodes_[y].l != kNil) nodes_[nodes_[y].l].p = x;
    nodes_[y].p = nodes_[x].p;
    if (nodes_[x].p == kNil)
      root_ = y;
    else if (x == nodes_[nodes_[x].p].l)
      nodes_[nodes_[x].p].l = y;
    else
      nodes_[nodes_[x].p].r = y;
    nodes_[y].l = x;
    nodes_[x].p = y;
  }
  void rotate_right(int32_t x) {
    const int32_t y = nodes_[x].l;
    nodes_[x].l = nodes_[y].r;
    if (nodes_[y].r != kNil) nodes_[nodes_[y].r].p = x;
    nodes_[y].p = nodes_[x].p;
    if (nodes_[x].p == kNil)
      root_ = y;
    else if (x == nodes_[nodes_[x].p].r)
      nodes_[nodes_[x].p].r = y;
    else
      nodes_[nodes_[x].p].l = y;
    nodes_[y].r = x;
    nodes_[x].p = y;
  }

  void insert_fixup(int32_t z) {
    while (red(nodes_[z].p)) {
      const int32_t p = nodes_[z].p, g = nodes_[p].p;
      if (p == nodes_[g].l) {
        const int32_t u = nodes_[g].r;
        if (red(u)) {
          nodes_[p].red = false;
          nodes_[u].red = false;
          nodes_[g].red = true;
          z = g;
        } else {
          if (z == nodes_[p].r) {
            z = p;
            rotate_left(z);
          }
          nodes_[nodes_[z].p].red = false;
          nodes_[nodes_[nodes_[z].p].p].red = true;
          rotate_right(nodes_[nodes_[z].p].p);
        }
      } else {
        const int32_t u = nodes_[g].l;
        if (red(u)) {
          nodes_[p].red = false;
          nodes_[u].red = false;
          nodes_[g].red = true;
          z = g;
        } else {
          if (z == nodes_[p].l) {
            z = p;
            rotate_right(z);
          }
          nodes_[nodes_[z].p].red = false;
          nodes_[nodes_[nodes_[z].p].p].red = true;
          rotate_left(nodes_[nodes_[z].p].p);
        }
      }
    }
    nodes_[root_].red = false;
  }

  // Replaces the subtree at u by the one at v (v may be nil); returns u's parent.
  int32_t transplant(int32_t u, int32_t v) {
    const int32_t up = nodes_[u].p;
    if (up == kNil)
      root_ = v;
    else if (u == nodes_[up].l)
      nodes_[up].l = v;
    else
      nodes_[up].r = v;
    if (v != kNil) nodes_[v].p = up;
    return up;
  }

  void erase(int32_t z) {
    int32_t y = z, x, xp;  // x replaces the removed position; xp is its parent (x may be nil)
    bool y_red = nodes_[y].red;
    if (nodes_[z].l == kNil) {
      x = nodes_[z].r;
      xp = transplant(z, x);
    } else if (nodes_[z].r == kNil) {
      x = nodes_[z].l;
      xp = transplant(z, x);
    } else {
      y = leftmost(nodes_[z].r);  // the successor takes z's place and colour
      y_red = nodes_[y].red;
      x = nodes_[y].r;
      if (nodes_[y].p == z) {
        xp = y;
      } else {
        xp = transplant(y, x);
        nodes_[y].r = nodes_[z].r;
        nodes_[nodes_[y].r].p = y;
      }
      transplant(z, y);
      nodes_[y].l = nodes_[z].l;
      nodes_[nodes_[y].l].p = y;
      nodes_[y].red = nodes_[z].red;
    }
    free_.push_back(z);
    size_--;
    if (!y_red) erase_fixup(x, xp);
  }

  void erase_fixup(int32_t x, int32_t xp) {
    while (x != root_ && !red(x)) {
      if (x == nodes_[xp].l) {
        int32_t w = nodes_[xp].r;
        if (red(w)) {
          nodes_[w].red = false;
          nodes_[xp].red = true;
          rotate_left(xp);
          w = nodes_[xp].r;
        }
        if (!red(nodes_[w].l) && !red(nodes_[w].r)) {
          nodes_[w].red = true;
          x = xp;
          xp = nodes_[x].p;
        } else {
          if (!red(nodes_[w].r)) {
            nodes_[nodes_[w].l].red = false;
            nodes_[w].red = true;
            rotate_right(w);
            w = nodes_[xp].r;
          }
          nodes_[w].red = nodes_[xp].red;
          nodes_[xp].red = false;
          if (nodes_[w].r != kNil) nodes_[nodes_[w].r].red = false;
          rotate_left(xp);
          x = root_;
          break;
        }
      } else {
        int32_t w = nodes_[xp].l;
        if (red(w)) {
          nodes_[w].red = false;
          nodes_[xp].red = true;
          rotate_right(xp);
          w = nodes_[xp].l;
        }
        if (!red(nodes_[w].r) && !red(nodes_[w].l)) {
          nodes_[w].red = true;
          x = xp;
          xp = nodes_[x].p;
        } else {
          if (!red(nodes_[w].l)) {
            nodes_[nodes_[w].r].red = false;
            nodes_[w].red = true;
            rotate_left(w);
            w = nodes_[xp].l;
          }
          nodes_[w].red = nodes_[xp].red;
          nodes_[xp].red = false;
          if (nodes_[w].l != kNil) nodes_[nodes_[w].l].red = false;
          rotate_right(xp);
          x = root_;
          break;
        }
      }
    }
    if (x != kNil) nodes_[x].red = false;
  }

  std::vector<Node> nodes_;
  std::vector<int32_t> free_;
  int32_t root_ = kNil;
  size_t size_ = 0;
};

}  // namespace smat
