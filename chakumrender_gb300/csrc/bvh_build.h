// bvh_build.h — host-side binned-SAH BVH builder and its flattened device layout.
#pragma once
#include <stdint.h>
#include <vector>

#include "../../include/ckr.h"

namespace ckr {

// Flattened wide BVH as uploaded to the device: the binary SAH tree collapsed
// into nodes of up to eight children with child boxes quantised to 8 bits per
// plane (after Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on
// GPUs Through Compressed Wide BVHs", HPG 2017).
//
// nodes: 20 words (80 bytes, five 16-byte words) per node, node 0 the root:
//   [0..2]  p.xyz (float bits): origin of the node's quantisation grid
//   [3]     ex | ey << 8 | ez << 16 | imask << 24.  e_a is the biased float
//           exponent of the grid step 2^(e_a - 127) on axis a; imask bit s is
//           set when slot s holds an interior child
//   [4]     child_base: index of the first interior child; the interior
//           children are stored contiguously in slot order
//   [5]     tri_base: index of the first triangle of the leaf children; their
//           triangles are stored contiguously in slot order
//   [6..7]  meta[8], one byte per slot: 0 = empty; interior = 0x20 | (24 + s);
//           leaf = unary(count) << 5 | (offset from tri_base), count 1..3
//   [8..9]  qlo.x[8]  [10..11] qhi.x[8]  [12..13] qlo.y[8]  [14..15] qhi.y[8]
//   [16..17] qlo.z[8] [18..19] qhi.z[8]
// The box of slot s on axis a is [p_a + qlo_a[s] 2^e_a, p_a + qhi_a[s] 2^e_a]
// in exact arithmetic, and it contains the child's exact FP32 box.  Slots are
// assigned per ray octant: slot o holds the child a ray of octant o (bit 2: dx
// < 0, bit 1: dy < 0, bit 0: dz < 0) should visit first.
//
// tris: 12 floats (three 16-byte words) per triangle in node order:
//   [0] A.xyz, input index (uint32 bits)   [1] B.xyz, 0   [2] C.xyz, 0
struct FlatBvh {
  std::vector<uint32_t> nodes;
  std::vector<float> tris;
  int32_t root = kEmptyRoot;  // 0, or kEmptyRoot when no triangle is indexed
  uint32_t nnodes = 0;        // wide nodes
  uint32_t nleaves = 0;       // leaf children (groups of 1..3 triangles)
  uint32_t max_depth = 0;     // levels of wide nodes (= traversal stack entries needed)
  uint32_t ntri_indexed = 0;
  uint32_t nnodes_binary = 0;  // interior nodes of the binary tree it was collapsed from
  static constexpr int32_t kEmptyRoot = (int32_t)0x80000000;  // no triangles
};

constexpr uint32_t kWideWords = 20;  // 32-bit words per wide node
constexpr uint32_t kWideLeafMax = 3;  // triangles per leaf child

// Builds over ntri triangles (9 floats each).  Triangles with a non-finite
// coordinate are left out: no ray can hit them (the reference's NaN-normal
// dummy triangle, src/prepareScene.cpp:241, never reports a hit either).
// Returns CKR_OK or an error code.
int build_bvh(const float *tri9, uint32_t ntri, const ckr_build_params &params, FlatBvh &out);

// Check of a flattened tree: child indices in range and each node reached once,
// leaf ranges tile the triangle array, every quantised box contains its child's
// exact box (checked in exact arithmetic), max_depth exact.  build_bvh runs it.
bool validate_bvh(const FlatBvh &b);

}  // namespace ckr
