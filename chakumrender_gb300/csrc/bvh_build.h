// bvh_build.h — host-side binned-SAH BVH builder and its flattened device layout.
#pragma once
#include <stdint.h>
#include <vector>

#include "../../include/ckr.h"

namespace ckr {

// Flattened BVH as uploaded to the device.
//
// nodes: 16 floats (four 16-byte words) per interior node, both child boxes:
//   [0] c0.lo.x c0.hi.x c0.lo.y c0.hi.y
//   [1] c1.lo.x c1.hi.x c1.lo.y c1.hi.y
//   [2] c0.lo.z c0.hi.z c1.lo.z c1.hi.z
//   [3] link0   link1   (int bits)  0 0
// A link >= 0 is an interior node index; a link < 0 is a leaf,
// ~link = (first_triangle << 3) | (count - 1).
//
// tris: 12 floats (three 16-byte words) per triangle in leaf order:
//   [0] A.xyz, input index (uint32 bits)   [1] B.xyz, 0   [2] C.xyz, 0
struct FlatBvh {
  std::vector<float> nodes;
  std::vector<float> tris;
  int32_t root = kEmptyRoot;  // link of the root (a leaf when the tree is one leaf)
  uint32_t nnodes = 0, nleaves = 0, max_depth = 0, ntri_indexed = 0;
  static constexpr int32_t kEmptyRoot = (int32_t)0x80000000;  // no triangles
};

inline int32_t leaf_link(uint32_t first, uint32_t count) {
  return (int32_t)~((first << 3) | (count - 1));
}

// Builds over ntri triangles (9 floats each).  Triangles with a non-finite
// coordinate are left out: no ray can hit them (the reference's NaN-normal
// dummy triangle, src/prepareScene.cpp:241, never reports a hit either).
// Returns CKR_OK or an error code.
int build_bvh(const float *tri9, uint32_t ntri, const ckr_build_params &params, FlatBvh &out);

// Structural check of a flattened tree (links in range, each node reached once,
// leaf ranges tile the triangle array, max_depth exact).  build_bvh runs it.
bool validate_bvh(const FlatBvh &b);

}  // namespace ckr
