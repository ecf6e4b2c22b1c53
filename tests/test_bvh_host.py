"""CPU checks of the SAH builder and the FP32 traversal logic (host replay of the device
algorithm, no GPU): structural validation runs inside the build, and the replayed
closest hits agree with the FP64 oracle under the same parity classification the GPU
tests use."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import ckr
from parity import classify

GOLD = Path(__file__).resolve().parent / "golden"


def replay(tri, rays, leaf=4, any_hit=False):
    L = ckr.lib()
    f = L.ckr_internal_replay
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p, C.c_void_p,
                  C.POINTER(C.c_double), C.POINTER(C.c_double)]
    f.restype = C.c_int
    tri = np.ascontiguousarray(tri, dtype=np.float32)
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    ids = np.empty(len(rays), dtype=np.uint32)
    t = np.empty(len(rays), dtype=np.float32)
    b, n = C.c_double(), C.c_double()
    st = f(tri.ctypes.data if len(tri) else None, len(tri), leaf, rays.ctypes.data, len(rays), int(any_hit),
           ids.ctypes.data, t.ctypes.data, C.byref(b), C.byref(n))
    assert st == 0, st
    return ids, t, b.value, n.value


def closest_rays(r):
    r = r.copy()
    r[:, 7] = 1e30
    return r


@pytest.mark.parametrize("name", ["trace_small", "trace_edges"])
@pytest.mark.parametrize("leaf", [1, 2, 4, 8])
def test_replay_matches_reference(name, leaf):
    g = np.load(GOLD / f"{name}.npz")
    ids, t, _, _ = replay(g["tri"], closest_rays(g["rays"]), leaf)
    c = classify(g["tri"], g["rays"], ids, t, g["ids"], g["t"])
    assert not c["bad"], c
    # trace_edges aims ~45% of its rays at shared edges and vertices on purpose.
    assert c["edge"] <= max(2, (0.1 if name == "trace_edges" else 1e-3) * len(g["rays"]))


def test_replay_medium_mesh_vs_oracle():
    tri = ckr.icosphere(6, 0.05, 6, 1)
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    rays = np.concatenate([ckr.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 96, 96),
                           ckr.rays_incoherent(lo, hi, 7, 8192)])
    ids, t, nodes, ntris = replay(tri, rays)
    oid, ot = O.OracleBvh(tri).closest(rays)
    c = classify(tri, rays, ids, t, oid, ot)
    assert not c["bad"], c
    assert c["edge"] <= 3
    # The reference's midpoint tree visits ~130 binary nodes per ray; the collapsed SAH
    # tree visits about 9 eight-wide nodes (measured 9.4) and 3.6 triangles.
    assert nodes < 14 and ntris < 6


def test_degenerate_inputs_build():
    bad = np.array([[1e6] * 9, [0] * 9, [np.nan] * 9], dtype=np.float32)
    rays = closest_rays(ckr.rays_incoherent([-1, -1, -1], [1, 1, 1], 1, 100))
    ids, _, _, _ = replay(bad, rays)
    assert np.all(ids == 0xFFFFFFFF)
    ids, _, _, _ = replay(np.zeros((0, 9), np.float32), rays)
    assert np.all(ids == 0xFFFFFFFF)
    # Many coincident triangles force splits of equal centroids; leaves stay <= 8.
    same = np.tile(np.array([[-1, -1, 0, 1, -1, 0, 0, 1, 0]], np.float32), (100, 1))
    r = closest_rays(np.array([[0, 0, 2, 0, 0, 0, -1, 1e30]], np.float32))
    ids, t, _, _ = replay(same, r)
    assert ids[0] < 100 and abs(t[0] - 2) < 1e-6


def test_axis_parallel_rays_stay_cheap():
    """Rays with exact zero direction components: the quantised slab test must keep
    those axes (a capped 1/d, not 0 x inf = NaN, which would drop the axis and send the
    ray through every node the other axes admit) and still find the oracle's hits."""
    tri = ckr.icosphere(6, 0.05, 6, 1)
    rng = np.random.default_rng(4)
    dirs = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [1, 1, 0], [0, -1, 1], [1, 0, -1], [-0.0, 0.0, -1]], np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    n = 4000
    o = rng.uniform(-1.5, 1.5, (n, 3)).astype(np.float32)
    o[: n // 4, 0] = 0.0  # origins on the coordinate planes too
    o[n // 4: n // 2, 1] = 0.0
    d = dirs[rng.integers(0, len(dirs), n)]
    rays = np.concatenate([o, np.zeros((n, 1), np.float32), d, np.full((n, 1), 1e30, np.float32)], 1)
    ids, t, nodes, ntris = replay(tri, rays)
    oid, ot = O.OracleBvh(tri).closest(rays)
    c = classify(tri, rays, ids, t, oid, ot)
    assert not c["bad"], c
    # Rays in a coordinate plane through the origin graze the mesh's edges that lie
    # in that plane (the icosphere has vertices with zero coordinates): boundary cases.
    assert c["edge"] <= 0.03 * n
    # A few nodes per ray, as for random rays; an axis lost to NaN costs hundreds.
    assert nodes < 20, nodes


def bvh_digest(tri, threads, leaf=0):
    L = ckr.lib()
    f = L.ckr_internal_bvh_digest
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]
    f.restype = C.c_int
    tri = np.ascontiguousarray(tri, dtype=np.float32)
    h, n = C.c_uint64(), C.c_uint32()
    assert f(tri.ctypes.data, len(tri), leaf, threads, C.byref(h), C.byref(n)) == 0
    return h.value, n.value


def test_build_is_the_same_on_any_number_of_threads():
    # 327,680 triangles: the plan and the writing of the wide nodes hand subtrees of
    # 32,768 or more triangles to other threads (the root's eight children hold
    # about 40,000 each), and the primitive setup splits into ranges.
    tri = ckr.icosphere(7, 0.05, 6, 1)
    one = bvh_digest(tri, 1)
    assert one[1] > 1000
    for threads in (2, 3, 8, 16):
        assert bvh_digest(tri, threads) == one, threads
    assert bvh_digest(tri, 5, leaf=1) == bvh_digest(tri, 1, leaf=1)
