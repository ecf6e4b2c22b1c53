// bvh_build.cpp — binned-SAH BVH builder (host, multi-threaded).
//
// Replaces the reference's centroid-midpoint, one-primitive-per-leaf build
// (src/bvhAccel.cpp:24-149).  The closest hit a ray reports does not depend
// on the tree (only ties in t can resolve differently), so any correct BVH is
// a drop-in; SAH trees visit far fewer nodes per ray.
//
// Algorithm: top-down binned SAH (Wald 2007, "On fast construction of
// SAH-based bounding volume hierarchies"), bins on all three centroid axes,
// costs C_trav = 1 and C_isect = 1 per triangle; large subtrees are built on
// separate threads.  The binary tree is then collapsed into eight-wide nodes
// with 8-bit quantised child boxes (Ylitie, Karras, Laine, HPG 2017; layout in
// bvh_build.h); the collapse's plan and the writing of the wide nodes run on
// several threads too, with the same output as a single thread.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>

namespace ckr {
namespace {

struct Box {
  float lo[3], hi[3];
  void reset() {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::numeric_limits<float>::infinity();
      hi[k] = -std::numeric_limits<float>::infinity();
    }
  }
  void grow(const Box &b) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], b.lo[k]);
      hi[k] = std::max(hi[k], b.hi[k]);
    }
  }
  void grow(const float *p) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], p[k]);
      hi[k] = std::max(hi[k], p[k]);
    }
  }
  float area() const {
    float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
    if (!(d0 >= 0.f) || !(d1 >= 0.f) || !(d2 >= 0.f)) return 0.f;
    return 2.f * (d0 * d1 + d1 * d2 + d2 * d0);
  }
};

struct Prim {
  Box box;
  float c[3];
  uint32_t id;
};

struct TNode {
  Box box;
  uint32_t left;   // index of left child in the node pool (right = left + 1)
  uint32_t begin;  // leaf: first prim index
  uint32_t count;  // leaf: prim count; 0 for interior
  uint32_t size;   // prims in the subtree
};

struct Builder {
  std::vector<Prim> prims;
  std::unique_ptr<TNode[]> pool;  // uninitialised: build() writes each node it allocates
  std::atomic<uint32_t> next{1};
  std::atomic<int> spare_threads{0};
  uint32_t max_leaf = 4, bins = 16, threads = 1;

  // Nodes of at least kParallelBin triangles (the top levels, where few subtrees
  // run at once) compute their centroid bounds, bins and child boxes on `threads`
  // threads, each over a contiguous range; the partial boxes and counts are merged,
  // and since min / max and counts do not depend on the order, the result is the
  // same as on one thread.
  static constexpr uint32_t kParallelBin = 1u << 18;

  template <class F>
  void ranges(uint32_t begin, uint32_t end, uint32_t parts, F f) {
    std::vector<std::thread> ts;
    for (uint32_t k = 1; k < parts; ++k)
      ts.emplace_back(f, k, begin + (uint32_t)((uint64_t)(end - begin) * k / parts),
                      begin + (uint32_t)((uint64_t)(end - begin) * (k + 1) / parts));
    f(0u, begin, begin + (uint32_t)((uint64_t)(end - begin) / parts));
    for (std::thread &t : ts) t.join();
  }

  uint32_t alloc2() { return next.fetch_add(2); }

  void make_leaf(TNode &n, uint32_t begin, uint32_t end) {
    n.begin = begin;
    n.count = end - begin;
    n.left = 0;
  }

  // Builds node `ni` over prims[begin, end) whose bounds are already in pool[ni].box.
  void build(uint32_t ni, uint32_t begin, uint32_t end) {
    TNode &node = pool[ni];
    uint32_t n = end - begin;
    node.size = n;
    if (n <= 1) {
      make_leaf(node, begin, end);
      return;
    }
    const uint32_t parts = n >= kParallelBin ? std::max(1u, std::min(threads, n >> 16)) : 1u;
    Box cb;
    cb.reset();
    if (parts > 1) {
      std::vector<Box> part(parts);
      ranges(begin, end, parts, [&](uint32_t k, uint32_t lo, uint32_t hi) {
        part[k].reset();
        for (uint32_t i = lo; i < hi; ++i) part[k].grow(prims[i].c);
      });
      for (const Box &b : part) cb.grow(b);
    } else {
      for (uint32_t i = begin; i < end; ++i) cb.grow(prims[i].c);
    }

    // Binned SAH over the three axes.
    const uint32_t B = bins;
    float best_cost = std::numeric_limits<float>::infinity();
    int best_axis = -1;
    uint32_t best_split = 0;
    Box bbox[64];
    uint32_t bcnt[64];
    float right_area[64];
    uint32_t right_cnt[64];
    // Large nodes: the bins of all three axes in one pass per thread.
    std::vector<Box> pbox;
    std::vector<uint32_t> pcnt;
    if (parts > 1) {
      pbox.resize((size_t)parts * 3 * B);
      pcnt.assign((size_t)parts * 3 * B, 0);
      ranges(begin, end, parts, [&](uint32_t k, uint32_t lo, uint32_t hi) {
        Box *bx = &pbox[(size_t)k * 3 * B];
        uint32_t *ct = &pcnt[(size_t)k * 3 * B];
        for (uint32_t b = 0; b < 3 * B; ++b) bx[b].reset();
        for (int axis = 0; axis < 3; ++axis) {
          const float ext = cb.hi[axis] - cb.lo[axis];
          if (!(ext > 0.f)) continue;
          const float scale = (float)B / ext;
          for (uint32_t i = lo; i < hi; ++i) {
            const uint32_t b = std::min(B - 1, (uint32_t)((prims[i].c[axis] - cb.lo[axis]) * scale));
            bx[axis * B + b].grow(prims[i].box);
            ct[axis * B + b]++;
          }
        }
      });
    }
    for (int axis = 0; axis < 3; ++axis) {
      float ext = cb.hi[axis] - cb.lo[axis];
      if (!(ext > 0.f)) continue;
      float scale = (float)B / ext;
      for (uint32_t b = 0; b < B; ++b) {
        bbox[b].reset();
        bcnt[b] = 0;
      }
      if (parts > 1) {
        for (uint32_t k = 0; k < parts; ++k)
          for (uint32_t b = 0; b < B; ++b) {
            bbox[b].grow(pbox[((size_t)k * 3 + axis) * B + b]);
            bcnt[b] += pcnt[((size_t)k * 3 + axis) * B + b];
          }
      } else {
        for (uint32_t i = begin; i < end; ++i) {
          uint32_t b = std::min(B - 1, (uint32_t)((prims[i].c[axis] - cb.lo[axis]) * scale));
          bbox[b].grow(prims[i].box);
          bcnt[b]++;
        }
      }
      Box acc;
      acc.reset();
      uint32_t cnt = 0;
      for (uint32_t b = B - 1; b > 0; --b) {
        acc.grow(bbox[b]);
        cnt += bcnt[b];
        right_area[b] = acc.area();
        right_cnt[b] = cnt;
      }
      acc.reset();
      cnt = 0;
      for (uint32_t b = 0; b + 1 < B; ++b) {
        acc.grow(bbox[b]);
        cnt += bcnt[b];
        if (cnt == 0 || right_cnt[b + 1] == 0) continue;
        float cost = acc.area() * (float)cnt + right_area[b + 1] * (float)right_cnt[b + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = axis;
          best_split = b + 1;
        }
      }
    }
    float parent_area = node.box.area();
    float leaf_cost = (float)n;
    float split_cost = parent_area > 0.f ? 1.f + best_cost / parent_area : std::numeric_limits<float>::infinity();
    if (n <= max_leaf && (best_axis < 0 || leaf_cost <= split_cost)) {
      make_leaf(node, begin, end);
      return;
    }
    uint32_t mid;
    if (best_axis >= 0) {
      float scale = (float)B / (cb.hi[best_axis] - cb.lo[best_axis]);
      float lo = cb.lo[best_axis];
      int axis = best_axis;
      Prim *m = std::partition(prims.data() + begin, prims.data() + end, [&](const Prim &p) {
        return std::min(B - 1, (uint32_t)((p.c[axis] - lo) * scale)) < best_split;
      });
      mid = (uint32_t)(m - prims.data());
      if (mid == begin || mid == end) mid = begin + n / 2;
    } else {
      mid = begin + n / 2;  // all centroids coincide: split the list in half
    }
    uint32_t l = alloc2();
    node.left = l;
    node.count = 0;
    TNode &L = pool[l], &R = pool[l + 1];
    L.box.reset();
    R.box.reset();
    if (parts > 1) {
      std::vector<Box> part(2 * (size_t)parts);
      ranges(begin, end, parts, [&](uint32_t k, uint32_t lo, uint32_t hi) {
        Box &l = part[2 * k], &r = part[2 * k + 1];
        l.reset();
        r.reset();
        for (uint32_t i = lo; i < hi; ++i) (i < mid ? l : r).grow(prims[i].box);
      });
      for (uint32_t k = 0; k < parts; ++k) {
        L.box.grow(part[2 * k]);
        R.box.grow(part[2 * k + 1]);
      }
    } else {
      for (uint32_t i = begin; i < mid; ++i) L.box.grow(prims[i].box);
      for (uint32_t i = mid; i < end; ++i) R.box.grow(prims[i].box);
    }
    if (n > 65536 && spare_threads.fetch_sub(1) > 0) {
      std::thread t([this, l, begin, mid] { build(l, begin, mid); });
      build(l + 1, mid, end);
      t.join();
      spare_threads.fetch_add(1);
    } else {
      if (n > 65536) spare_threads.fetch_add(1);
      build(l, begin, mid);
      build(l + 1, mid, end);
    }
  }
};

// Exact position of a quantised plane, p + q 2^e.  Exact in double: p and the
// bound it is compared with are floats within the node's extent of each other
// and q 2^e has at most 8 significant bits.
inline double plane(float p, uint32_t q, int e) { return (double)p + std::ldexp((double)q, e); }

// One child of a wide node under construction: an interior node of the binary
// tree that becomes a wide node, or a leaf of 1..3 triangles.
struct Entry {
  Box box;
  uint32_t tnode;         // interior: binary-tree node
  uint32_t begin, count;  // leaf: prims[begin, begin + count); count 0 for interior
};

// SAH cost model of the collapse: a wide-node visit costs kCostNode, a triangle
// test kCostPrim, each weighted by the surface area of the box whose hit leads to
// it.  A triangle test takes about a third of the instructions of a node visit,
// but the traversal tests one triangle per step while lanes of the warp visit
// nodes, so on the device it costs about as much as a visit: sweeping kCostPrim
// over 0.3 .. 1.5 on the 1.3M-triangle workload, 0.3 was 5 % slower and 1.0 .. 1.5
// equal.
constexpr float kCostNode = 1.0f, kCostPrim = 1.0f;

// Subtrees of at least this many triangles are handed to another thread while
// spare threads remain (plan and emission alike).
constexpr uint32_t kParallelPrims = 1u << 15;

// Optimal collapse of the binary tree (the dynamic programme of Ylitie et al.
// 2017).  For binary node n, cost[8n + j - 1] is the least cost of spreading n's
// subtree over at most j slots of the wide node above it: n itself in one slot
// (as a leaf of <= leaf_max triangles or as a wide node of its own), or the
// slots shared between its two children.  wide[8n + j - 1] counts the wide nodes
// that choice creates, so that every wide subtree's place in the output is known
// before it is written.
struct Plan {
  // Every entry of a binary node is written when the node is planned, so the
  // arrays are left uninitialised (a few hundred MB at a million triangles).
  std::unique_ptr<float[]> cost;
  std::unique_ptr<uint32_t[]> wide;
  std::unique_ptr<uint8_t[]> split;   // per (n, j): 0 = n takes one slot, k = k slots to the left child
  std::unique_ptr<uint8_t[]> leaf;    // n in one slot is a leaf (else a wide node)
  std::unique_ptr<uint8_t[]> wsplit;  // n as a wide node: slots of its left child (right: 8 - wsplit)
  std::unique_ptr<uint32_t[]> begin, count;  // n's triangles: prims[begin, begin + count)

  explicit Plan(uint32_t N)
      : cost(new float[(size_t)N * 8]), wide(new uint32_t[(size_t)N * 8]), split(new uint8_t[(size_t)N * 8]),
        leaf(new uint8_t[N]), wsplit(new uint8_t[N]), begin(new uint32_t[N]), count(new uint32_t[N]) {}

  // Wide nodes below interior binary node n made a wide node (its descendants).
  uint32_t below(const Builder &b, uint32_t n) const {
    const uint32_t L = b.pool[n].left;
    return wide[(size_t)L * 8 + wsplit[n] - 1] + wide[(size_t)(L + 1) * 8 + (8 - wsplit[n]) - 1];
  }
};

// The plan's entries of binary node i from those of its children.
void plan_node(const Builder &b, uint32_t leaf_max, Plan &p, uint32_t i) {
  const TNode &n = b.pool[i];
  float *d = &p.cost[(size_t)i * 8];
  uint32_t *w = &p.wide[(size_t)i * 8];
  const float area = n.box.area();
  uint8_t *sp = &p.split[(size_t)i * 8];
  if (n.count) {  // binary leaf (one triangle: the binary tree is built with leaf size 1)
    p.begin[i] = n.begin;
    p.count[i] = n.count;
    p.leaf[i] = 1;
    p.wsplit[i] = 1;
    for (int j = 0; j < 8; ++j) {
      d[j] = area * (float)n.count * kCostPrim;
      w[j] = 0;
      sp[j] = 0;
    }
    return;
  }
  const uint32_t L = n.left, R = L + 1;
  p.begin[i] = p.begin[L];
  p.count[i] = p.count[L] + p.count[R];
  const float *dl = &p.cost[(size_t)L * 8], *dr = &p.cost[(size_t)R * 8];
  const uint32_t *wl = &p.wide[(size_t)L * 8], *wr = &p.wide[(size_t)R * 8];
  float best = std::numeric_limits<float>::infinity();
  int bk = 1;
  for (int k = 1; k <= 7; ++k) {
    const float c = dl[k - 1] + dr[8 - k - 1];
    if (c < best) {
      best = c;
      bk = k;
    }
  }
  const float c_wide = area * kCostNode + best;
  const float c_leaf = p.count[i] <= leaf_max ? area * (float)p.count[i] * kCostPrim
                                              : std::numeric_limits<float>::infinity();
  const float c1 = std::min(c_leaf, c_wide);
  p.leaf[i] = c_leaf <= c_wide;
  p.wsplit[i] = (uint8_t)bk;
  d[0] = c1;
  w[0] = p.leaf[i] ? 0u : 1u + wl[bk - 1] + wr[8 - bk - 1];
  sp[0] = 0;
  for (int j = 2; j <= 8; ++j) {
    float bj = c1;
    int sj = 0;
    for (int k = 1; k < j; ++k) {
      const float c = dl[k - 1] + dr[j - k - 1];
      if (c < bj) {
        bj = c;
        sj = k;
      }
    }
    d[j - 1] = bj;
    w[j - 1] = sj ? wl[sj - 1] + wr[j - sj - 1] : w[0];
    sp[j - 1] = (uint8_t)sj;
  }
}

// Plans the subtree of binary node `root`, children before parents.  While spare
// threads remain, a large subtree's left half goes to another thread (joined
// before the node itself is planned); the rest is an explicit-stack post-order.
void plan_subtree(const Builder &b, uint32_t leaf_max, Plan &p, uint32_t root, std::atomic<int> &spare) {
  const TNode &r = b.pool[root];
  if (r.count == 0 && r.size >= kParallelPrims && spare.fetch_sub(1) > 0) {
    std::thread t([&b, leaf_max, &p, &r, &spare] { plan_subtree(b, leaf_max, p, r.left, spare); });
    plan_subtree(b, leaf_max, p, r.left + 1, spare);
    t.join();
    spare.fetch_add(1);
    plan_node(b, leaf_max, p, root);
    return;
  }
  if (r.count == 0 && r.size >= kParallelPrims) spare.fetch_add(1);
  struct Item {
    uint32_t node;
    bool expanded;
  };
  std::vector<Item> stack{{root, false}};
  while (!stack.empty()) {
    const Item it = stack.back();
    stack.pop_back();
    const TNode &n = b.pool[it.node];
    if (it.expanded || n.count) {
      plan_node(b, leaf_max, p, it.node);
      continue;
    }
    stack.push_back({it.node, true});
    stack.push_back({n.left + 1, false});
    stack.push_back({n.left, false});
  }
}

// The slot children of binary node n spread over at most j slots, appended to
// kids[0 .. nk).
void gather(const Builder &b, const Plan &p, uint32_t n, uint32_t j, Entry *kids, int &nk) {
  const uint32_t s = p.split[(size_t)n * 8 + j - 1];
  if (s == 0) {
    if (p.leaf[n])
      kids[nk++] = {b.pool[n].box, 0, p.begin[n], p.count[n]};
    else
      kids[nk++] = {b.pool[n].box, n, 0, 0};
    return;
  }
  gather(b, p, b.pool[n].left, s, kids, nk);
  gather(b, p, b.pool[n].left + 1, j - s, kids, nk);
}

// Float to an unsigned key with the same order (no NaN); -0 is taken as +0.
inline uint32_t order_key(float f) {
  uint32_t u;
  f += 0.0f;
  std::memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Writes the wide tree into out.nodes / out.tris.  The output order is the one a
// depth-first emission gives: a node's interior children get consecutive indices
// when the node is written, the first slot's subtree is written next, and a node's
// leaf triangles are appended when it is written.  With the plan's wide-node counts
// every subtree's first node index, first child index and first triangle are known
// up front, so subtrees are written by several threads into disjoint ranges.
struct Emitter {
  const Builder &b;
  const Plan &p;
  const float *tri9;
  FlatBvh &out;
  std::atomic<int> &spare;
  std::atomic<uint32_t> nleaves{0}, max_depth{0};

  struct Work {
    uint32_t tnode, index, child_base, tri_base, depth;
  };

  // Writes the subtree of `root` (a wide node) and everything below it.
  void run(Work root) {
    std::vector<Work> work{root};
    std::vector<std::thread> threads;
    uint32_t leaves = 0, depth_max = 0;
    while (!work.empty()) {
      const Work wk = work.back();
      work.pop_back();
      depth_max = std::max(depth_max, wk.depth);
      Entry kids[8];
      int nk = 0;
      const TNode &tn = b.pool[wk.tnode];
      if (tn.count > 0) {
        kids[nk++] = {tn.box, 0, tn.begin, tn.count};  // the whole tree is one triangle
      } else {
        gather(b, p, tn.left, p.wsplit[wk.tnode], kids, nk);
        gather(b, p, tn.left + 1, 8 - p.wsplit[wk.tnode], kids, nk);
      }
      int slot_kid[8];
      uint32_t nint = 0, ntri = 0;
      write_node(wk, kids, nk, slot_kid, nint, ntri, leaves);
      // Children in slot order: indices child_base + k, their own children and
      // triangles after everything written before them.
      uint32_t cb = wk.child_base + nint, tb = wk.tri_base + ntri, k = 0;
      Work child[8];
      for (int slot = 0; slot < 8; ++slot) {
        if (slot_kid[slot] < 0 || kids[slot_kid[slot]].count != 0) continue;
        const uint32_t c = kids[slot_kid[slot]].tnode;
        child[k] = {c, wk.child_base + k, cb, tb, wk.depth + 1};
        cb += p.below(b, c);
        tb += p.count[c];
        ++k;
      }
      for (uint32_t i = k; i-- > 0;) {
        if (b.pool[child[i].tnode].size >= kParallelPrims && spare.fetch_sub(1) > 0) {
          threads.emplace_back([this, w = child[i]] {
            run(w);
            spare.fetch_add(1);
          });
          continue;
        }
        if (b.pool[child[i].tnode].size >= kParallelPrims) spare.fetch_add(1);
        work.push_back(child[i]);
      }
    }
    for (std::thread &t : threads) t.join();
    nleaves.fetch_add(leaves);
    uint32_t m = max_depth.load();
    while (m < depth_max && !max_depth.compare_exchange_weak(m, depth_max)) {
    }
  }

  // One wide node: slot assignment, quantised boxes, meta bytes, its leaf
  // children's triangles.  Out: slot -> kid (-1: empty), interior children and
  // triangles written.
  void write_node(const Work &wk, const Entry *kids, int nk, int *slot_kid, uint32_t &nint, uint32_t &ntri,
                  uint32_t &leaves) {
    // Node box and quantisation grid.
    Box nb;
    nb.reset();
    for (int k = 0; k < nk; ++k) nb.grow(kids[k].box);
    float centre[3];
    for (int a = 0; a < 3; ++a) centre[a] = 0.5f * nb.lo[a] + 0.5f * nb.hi[a];
    // Children go to slots by a greedy assignment on cost(child, slot) = (centroid
    // - node centre) . dir(slot), dir = the octant's signs, cheapest pair first
    // (ties: lower child, then lower slot), so that slot o holds the child nearest
    // the start of rays travelling in octant o.
    uint64_t keys[64];
    int np = 0;
    for (int k = 0; k < nk; ++k) {
      float c[3];
      for (int a = 0; a < 3; ++a) c[a] = 0.5f * kids[k].box.lo[a] + 0.5f * kids[k].box.hi[a] - centre[a];
      for (int slot = 0; slot < 8; ++slot) {
        const float cost = ((slot & 4) ? -c[0] : c[0]) + ((slot & 2) ? -c[1] : c[1]) + ((slot & 1) ? -c[2] : c[2]);
        keys[np++] = (uint64_t)order_key(cost) << 32 | (uint32_t)(k * 8 + slot);
      }
    }
    std::sort(keys, keys + np);
    bool placed[8] = {false, false, false, false, false, false, false, false};
    for (int s = 0; s < 8; ++s) slot_kid[s] = -1;
    for (int i = 0; i < np; ++i) {
      const int kid = (int)((keys[i] & 0xffffffffu) >> 3), slot = (int)(keys[i] & 7u);
      if (slot_kid[slot] < 0 && !placed[kid]) {
        slot_kid[slot] = kid;
        placed[kid] = true;
      }
    }
    uint32_t w[kWideWords] = {};
    std::memcpy(&w[0], &nb.lo[0], 12);
    int e[3];
    for (int a = 0; a < 3; ++a) {
      const double p0 = nb.lo[a], hi = nb.hi[a], ext = hi - p0;
      int ex = -126;
      if (ext > 0.0) {
        std::frexp(ext / 255.0, &ex);  // 2^ex > ext / 255
        while (ex > -126 && p0 + 255.0 * std::ldexp(1.0, ex - 1) >= hi) --ex;
        while (p0 + 255.0 * std::ldexp(1.0, ex) < hi) ++ex;
      }
      e[a] = std::max(-126, std::min(127, ex));
      w[3] |= (uint32_t)(e[a] + 127) << (8 * a);
    }
    uint8_t meta[8] = {}, q[6][8] = {};
    uint32_t imask = 0;
    nint = ntri = 0;
    for (int slot = 0; slot < 8; ++slot) {
      if (slot_kid[slot] < 0) continue;
      const Entry &c = kids[slot_kid[slot]];
      for (int a = 0; a < 3; ++a) {
        const double p0 = nb.lo[a], step = std::ldexp(1.0, e[a]);
        double lo = std::floor(((double)c.box.lo[a] - p0) / step), hi = std::ceil(((double)c.box.hi[a] - p0) / step);
        uint32_t ql = (uint32_t)std::max(0.0, std::min(255.0, lo)), qh = (uint32_t)std::max(0.0, std::min(255.0, hi));
        while (ql > 0 && plane(nb.lo[a], ql, e[a]) > (double)c.box.lo[a]) --ql;
        while (qh < 255 && plane(nb.lo[a], qh, e[a]) < (double)c.box.hi[a]) ++qh;
        q[2 * a][slot] = (uint8_t)ql;
        q[2 * a + 1][slot] = (uint8_t)qh;
      }
      if (c.count == 0) {
        imask |= 1u << slot;
        meta[slot] = (uint8_t)(0x38 + slot);
        ++nint;
      } else {
        meta[slot] = (uint8_t)((((1u << c.count) - 1u) << 5) | ntri);
        for (uint32_t i = c.begin; i < c.begin + c.count; ++i) {
          const float *t = tri9 + 9 * (size_t)b.prims[i].id;
          float *rec = &out.tris[(size_t)(wk.tri_base + ntri++) * 12];
          const float r[12] = {t[0], t[1], t[2], 0.f, t[3], t[4], t[5], 0.f, t[6], t[7], t[8], 0.f};
          std::memcpy(rec, r, sizeof(r));
          std::memcpy(&rec[3], &b.prims[i].id, 4);
        }
        ++leaves;
      }
    }
    w[3] |= imask << 24;
    w[4] = wk.child_base;
    w[5] = wk.tri_base;
    std::memcpy(&w[6], meta, 8);
    std::memcpy(&w[8], q, 48);
    std::memcpy(&out.nodes[(size_t)wk.index * kWideWords], w, sizeof(w));
  }
};

void collapse(const Builder &b, const float *tri9, uint32_t leaf_max, uint32_t threads, FlatBvh &out) {
  const uint32_t n = (uint32_t)b.prims.size();
  const uint32_t N = b.next.load();
  Plan plan(N);
  std::atomic<int> spare{(int)threads - 1};
  plan_subtree(b, leaf_max, plan, 0, spare);
  out.nnodes_binary = 0;
  for (uint32_t i = 0; i < N; ++i)
    if (b.pool[i].count == 0) out.nnodes_binary++;
  out.root = 0;
  out.nnodes = b.pool[0].count ? 1u : 1u + plan.below(b, 0);
  out.nodes.assign((size_t)out.nnodes * kWideWords, 0u);
  out.tris.assign((size_t)n * 12, 0.f);
  Emitter em{b, plan, tri9, out, spare};
  em.run({0, 0, 1, 0, 1});
  out.nleaves = em.nleaves.load();
  out.max_depth = em.max_depth.load();
}

}  // namespace

int build_bvh(const float *tri9, uint32_t ntri, const ckr_build_params &params, FlatBvh &out) {
  out = FlatBvh();
  Builder b;
  // The binary tree splits down to single triangles; the collapse chooses the
  // wide tree's leaves (at most leaf_max <= kWideLeafMax triangles each).
  const uint32_t req = params.max_leaf_size ? params.max_leaf_size : kWideLeafMax;
  b.bins = params.sah_bins ? params.sah_bins : 16;
  if (req < 1 || req > 8 || b.bins < 4 || b.bins > 64) return CKR_ERR_INVALID_ARGUMENT;
  const uint32_t leaf_max = std::min(req, kWideLeafMax);
  b.max_leaf = 1;
  unsigned hw = std::thread::hardware_concurrency();
  uint32_t threads = params.threads ? params.threads : (hw ? hw : 1);
  b.spare_threads = (int)threads - 1;
  b.threads = threads;

  // Primitive boxes, by contiguous ranges on all threads; the ranges' finite
  // triangles are then concatenated in input order.
  const uint32_t parts = std::max(1u, std::min(threads, ntri / 65536));
  std::vector<std::vector<Prim>> part(parts);
  auto setup = [&](uint32_t k) {
    const uint32_t lo = (uint32_t)((uint64_t)ntri * k / parts), hi = (uint32_t)((uint64_t)ntri * (k + 1) / parts);
    std::vector<Prim> &v = part[k];
    v.reserve(hi - lo);
    for (uint32_t i = lo; i < hi; ++i) {
      const float *t = tri9 + 9 * (size_t)i;
      bool finite = true;
      for (int c = 0; c < 9; ++c) finite = finite && std::isfinite(t[c]);
      if (!finite) continue;
      Prim p;
      p.box.reset();
      p.box.grow(t);
      p.box.grow(t + 3);
      p.box.grow(t + 6);
      for (int c = 0; c < 3; ++c) p.c[c] = 0.5f * p.box.lo[c] + 0.5f * p.box.hi[c];
      p.id = i;
      v.push_back(p);
    }
  };
  {
    std::vector<std::thread> ts;
    for (uint32_t k = 1; k < parts; ++k) ts.emplace_back(setup, k);
    setup(0);
    for (std::thread &t : ts) t.join();
  }
  size_t total = 0;
  for (const auto &v : part) total += v.size();
  b.prims.reserve(total);
  for (auto &v : part) {
    b.prims.insert(b.prims.end(), v.begin(), v.end());
    std::vector<Prim>().swap(v);
  }
  uint32_t n = (uint32_t)b.prims.size();
  out.ntri_indexed = n;
  if (n == 0) {
    out.root = FlatBvh::kEmptyRoot;
    return CKR_OK;
  }
  if (n >= (1u << 28)) return CKR_ERR_TOO_LARGE;
  b.pool.reset(new TNode[2 * (size_t)n + 1]);
  b.pool[0].box.reset();
  for (const Prim &p : b.prims) b.pool[0].box.grow(p.box);
  b.build(0, 0, n);

  collapse(b, tri9, leaf_max, threads, out);
  return validate_bvh(out) ? CKR_OK : CKR_ERR_INVALID_ARGUMENT;
}

bool validate_bvh(const FlatBvh &b) {
  const uint32_t ntri = (uint32_t)(b.tris.size() / 12);
  if (b.root == FlatBvh::kEmptyRoot) return ntri == 0 && b.nnodes == 0 && b.nodes.empty();
  if (b.root != 0 || b.nnodes == 0 || b.nodes.size() != (size_t)b.nnodes * kWideWords) return false;
  std::vector<uint32_t> level(b.nnodes, 0);
  std::vector<uint8_t> covered(ntri, 0);
  level[0] = 1;
  uint32_t depth_max = 0, leaves = 0;
  // Top-down: children lie after their parent, so one pass in index order sees
  // every parent before its children.
  for (uint32_t i = 0; i < b.nnodes; ++i) {
    if (level[i] == 0) return false;  // unreachable node
    depth_max = std::max(depth_max, level[i]);
    const uint32_t *w = &b.nodes[(size_t)i * kWideWords];
    const uint32_t imask = w[3] >> 24, child_base = w[4], tri_base = w[5];
    uint8_t meta[8];
    std::memcpy(meta, &w[6], 8);
    uint32_t nint = 0;
    for (uint32_t slot = 0; slot < 8; ++slot) {
      const uint32_t m = meta[slot];
      const bool inner = (imask >> slot) & 1u;
      if (inner) {
        if (m != 0x38u + slot) return false;
        uint64_t c = (uint64_t)child_base + nint++;
        if (c >= b.nnodes || c <= i || level[c] != 0) return false;
        level[c] = level[i] + 1;
      } else if (m != 0) {
        const uint32_t bits = m >> 5, off = m & 31u;
        const uint32_t cnt = bits == 1 ? 1 : bits == 3 ? 2 : bits == 7 ? 3 : 0;
        if (cnt == 0 || off + cnt > 24 || (uint64_t)tri_base + off + cnt > ntri) return false;
        for (uint32_t k = tri_base + off; k < tri_base + off + cnt; ++k) {
          if (covered[k]) return false;
          covered[k] = 1;
        }
        leaves++;
      }
    }
  }
  for (uint8_t c : covered)
    if (!c) return false;
  // Bottom-up, deepest level first (a node's children lie one level below it), the
  // nodes of a level on several threads: exact boxes, and each one inside its
  // quantised slot box.
  std::vector<float> box((size_t)b.nnodes * 6);
  std::vector<uint32_t> order(b.nnodes), first(depth_max + 2, 0);
  for (uint32_t i = 0; i < b.nnodes; ++i) first[level[i] + 1]++;
  for (uint32_t l = 1; l <= depth_max + 1; ++l) first[l] += first[l - 1];
  {
    std::vector<uint32_t> fill(first.begin(), first.end() - 1);
    for (uint32_t i = 0; i < b.nnodes; ++i) order[fill[level[i]]++] = i;
  }
  std::atomic<bool> ok{true};
  auto check = [&](uint32_t i) -> bool {
    const uint32_t *w = &b.nodes[(size_t)i * kWideWords];
    const uint32_t imask = w[3] >> 24, child_base = w[4], tri_base = w[5];
    uint8_t meta[8], q[6][8];
    std::memcpy(meta, &w[6], 8);
    std::memcpy(q, &w[8], 48);
    float p[3];
    std::memcpy(p, &w[0], 12);
    int e[3];
    for (int a = 0; a < 3; ++a) e[a] = (int)((w[3] >> (8 * a)) & 0xffu) - 127;
    float *nb = &box[(size_t)i * 6];
    for (int a = 0; a < 3; ++a) {
      nb[a] = std::numeric_limits<float>::infinity();
      nb[3 + a] = -std::numeric_limits<float>::infinity();
    }
    uint32_t nint = 0;
    for (uint32_t slot = 0; slot < 8; ++slot) {
      const uint32_t m = meta[slot];
      if (m == 0) continue;
      float cb[6];
      if ((imask >> slot) & 1u) {
        std::memcpy(cb, &box[(size_t)(child_base + nint++) * 6], sizeof(cb));
      } else {
        const uint32_t bits = m >> 5, off = m & 31u, cnt = bits == 1 ? 1 : bits == 3 ? 2 : 3;
        for (int a = 0; a < 3; ++a) {
          cb[a] = std::numeric_limits<float>::infinity();
          cb[3 + a] = -std::numeric_limits<float>::infinity();
        }
        for (uint32_t k = tri_base + off; k < tri_base + off + cnt; ++k)
          for (int v = 0; v < 3; ++v)
            for (int a = 0; a < 3; ++a) {
              float x = b.tris[(size_t)k * 12 + 4 * v + a];
              cb[a] = std::min(cb[a], x);
              cb[3 + a] = std::max(cb[3 + a], x);
            }
      }
      for (int a = 0; a < 3; ++a) {
        if (plane(p[a], q[2 * a][slot], e[a]) > (double)cb[a]) return false;
        if (plane(p[a], q[2 * a + 1][slot], e[a]) < (double)cb[3 + a]) return false;
        nb[a] = std::min(nb[a], cb[a]);
        nb[3 + a] = std::max(nb[3 + a], cb[3 + a]);
      }
    }
    return true;
  };
  const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
  for (uint32_t l = depth_max; l >= 1; --l) {
    const uint32_t lo = first[l], hi = first[l + 1], cnt = hi - lo;
    const uint32_t parts = std::max(1u, std::min(hw, cnt / 4096));
    auto run = [&](uint32_t k) {
      const uint32_t a = lo + (uint32_t)((uint64_t)cnt * k / parts), z = lo + (uint32_t)((uint64_t)cnt * (k + 1) / parts);
      for (uint32_t j = a; j < z && ok.load(std::memory_order_relaxed); ++j)
        if (!check(order[j])) ok = false;
    };
    std::vector<std::thread> ts;
    for (uint32_t k = 1; k < parts; ++k) ts.emplace_back(run, k);
    run(0);
    for (std::thread &t : ts) t.join();
    if (!ok) return false;
  }
  return depth_max == b.max_depth && leaves == b.nleaves;
}

}  // namespace ckr
