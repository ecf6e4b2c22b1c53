"""Hit-id parity classification between the FP32 traversal and the FP64 oracle.

The bar: hit ids bit-exact, except
  (a) ties in t: two different triangles hit at distances within 1e-5 relative;
  (b) boundary rays, where FP32 and FP64 legitimately disagree about whether a given
      triangle is hit:
        - the ray meets the plane of the triangle in question within EDGE_ABS (a few
          FP32 ulps, scaled by the coordinates' magnitude) of its boundary -- grazing an
          edge or vertex, including the gaps the reference's non-watertight FP64 test
          leaves at shared vertices;
        - |d.n| within 1% of the reference's near-parallel threshold 1e-5;
        - the hit lies at |t| <= 1e-5 (the ray starts on that surface and the sign of
          t ~ 0 decides).
Class (b) is bounded by the callers to a small count.  Anything else is "bad".
"""
from __future__ import annotations

import numpy as np

import oracle as O

MISS = 0xFFFFFFFF
T_REL = 1e-5
EDGE_ABS = 2e-6


def _boundary(tri9, ray, k, t_hit):
    """True if triangle k is a boundary case for this ray (see module docstring)."""
    if abs(t_hit) <= 1e-5:
        return True
    dist, tp = O.tri_edge_distance(tri9[k], ray)
    scale = max(1.0, float(np.abs(ray[:3]).max()), abs(tp) if np.isfinite(tp) else 1.0)
    if abs(dist) <= EDGE_ABS * scale:
        return True
    _, _, dn = O.tri_intersect(tri9[k], ray)
    return abs(dn - 1e-5) <= 1e-7


def classify(tri9, rays, gpu_id, gpu_t, ref_id, ref_t):
    """Returns a dict of counts and the indices of unexplained mismatches."""
    gpu_id = np.asarray(gpu_id, dtype=np.uint32)
    ref_id = np.asarray(ref_id, dtype=np.uint32)
    out = {"n": len(rays), "exact": 0, "tie": 0, "edge": 0, "t_off": 0, "bad": []}
    same = gpu_id == ref_id
    hit = same & (ref_id != MISS)
    tol = T_REL * np.maximum(np.abs(ref_t), 1.0)
    t_ok = np.abs(gpu_t.astype(np.float64) - ref_t) <= tol
    out["exact"] = int(np.sum(same & ~hit) + np.sum(hit & t_ok))
    for i in np.nonzero(hit & ~t_ok)[0]:
        out["t_off"] += 1
        out["bad"].append(int(i))
    for i in np.nonzero(~same)[0]:
        g, r = int(gpu_id[i]), int(ref_id[i])
        if g != MISS and r != MISS and abs(float(gpu_t[i]) - ref_t[i]) <= T_REL * max(abs(ref_t[i]), 1.0):
            out["tie"] += 1
            continue
        ok = (g != MISS and _boundary(tri9, rays[i], g, float(gpu_t[i]))) or \
             (r != MISS and _boundary(tri9, rays[i], r, float(ref_t[i])))
        if ok:
            out["edge"] += 1
        else:
            out["bad"].append(int(i))
    return out
