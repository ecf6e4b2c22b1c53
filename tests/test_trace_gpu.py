"""GPU parity of the traversal kernels (ckr_trace_closest / ckr_trace_any) against the
reference's answers (golden fixtures) and the FP64 oracle, through the C ABI."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import ckr
from parity import MISS, _boundary, classify

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def closest_rays(rays):
    r = np.array(rays, dtype=np.float32, copy=True)
    r[:, 7] = 1e30
    return r


def trace_device(torch, scene, rays):
    """Device-buffer entry points on torch tensors; returns numpy results."""
    d_rays = torch.from_numpy(np.ascontiguousarray(rays)).cuda()
    n = len(rays)
    ids = torch.empty(n, dtype=torch.int32, device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    occ = torch.empty(n, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    scene.trace_closest(d_rays.data_ptr(), n, ids.data_ptr(), t.data_ptr(), s)
    scene.trace_any(d_rays.data_ptr(), n, occ.data_ptr(), s)
    assert scene.check_device(s) == 0
    return ids.cpu().numpy().view(np.uint32), t.cpu().numpy(), occ.cpu().numpy()


def assert_parity(tri, rays, gid, gt, rid, rt, max_edge_frac):
    c = classify(tri, rays, gid, gt, rid, rt)
    assert not c["bad"], (c, [(i, int(gid[i]), float(gt[i]), int(rid[i]), float(rt[i])) for i in c["bad"][:10]])
    assert c["edge"] <= max(2, max_edge_frac * len(rays)), c
    return c


@pytest.mark.parametrize("name,edge_frac", [("trace_small", 1e-3), ("trace_edges", 0.1)])
def test_golden_closest_and_any(torch_cuda, name, edge_frac):
    g = np.load(GOLD / f"{name}.npz")
    tri, rays = g["tri"], g["rays"]
    for leaf in (1, 4, 8):
        scene = ckr.Scene(tri, max_leaf_size=leaf)
        gid, gt, _ = trace_device(torch_cuda, scene, closest_rays(rays))
        assert_parity(tri, rays, gid, gt, g["ids"], g["t"], edge_frac)
        _, _, occ = trace_device(torch_cuda, scene, rays)
        # Any-hit agrees with shadow() except where the closest hit is a tie/edge case at tmax.
        diff = np.nonzero(occ != g["occluded"])[0]
        ob = O.OracleBvh(tri)
        oid, ot = ob.closest(closest_rays(rays))
        for i in diff:
            near_tmax = abs(ot[i] - rays[i, 7]) <= 1e-5 * max(1.0, rays[i, 7])
            # The occluder (GPU's first hit or the oracle's closest) is a boundary case.
            gi = int(gid[i])
            on_edge = (oid[i] != MISS and _boundary(tri, rays[i], int(oid[i]), float(ot[i]))) or \
                      (gi != MISS and _boundary(tri, rays[i], gi, float(gt[i])))
            assert near_tmax or on_edge, (i, occ[i], g["occluded"][i], ot[i], rays[i])
        assert len(diff) <= max(2, edge_frac * len(rays))


def test_host_entry_points_match_device(torch_cuda):
    g = np.load(GOLD / "trace_small.npz")
    scene = ckr.Scene(g["tri"])
    rays = closest_rays(g["rays"])
    gid, gt, _ = trace_device(torch_cuda, scene, rays)
    hid, ht = scene.trace_closest_host(rays)
    assert np.array_equal(gid, hid) and np.array_equal(gt, ht)
    _, _, occ = trace_device(torch_cuda, scene, g["rays"])
    assert np.array_equal(occ, scene.trace_any_host(g["rays"]))


def test_host_entry_points_with_pinned_buffers(torch_cuda):
    """Rays in pinned memory are read in place by the kernels (no upload); a view
    that is not 16-byte aligned goes through the staged upload.  Both agree with the
    device-buffer entry points, over several chunks of the host pipeline."""
    torch = torch_cuda
    tri = ckr.icosphere(5, 0.05, 6, 1)
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    rays = ckr.rays_incoherent(lo, hi, 11, (3 << 20) + 12345, 0.05, 2.0)
    scene = ckr.Scene(tri)
    gid, gt, gocc = trace_device(torch, scene, closest_rays(rays))
    _, _, gocc = trace_device(torch, scene, rays)
    n = len(rays)
    L = ckr.lib()
    for shift in (0, 1):  # shift 1: the rays start 4 bytes into the pinned block
        flat = torch.empty(n * 8 + 4, dtype=torch.float32).pin_memory()
        h_rays = flat[shift:shift + n * 8].view(n, 8)
        h_rays.copy_(torch.from_numpy(closest_rays(rays)))
        h_ids = torch.zeros(n, dtype=torch.int32).pin_memory()
        h_t = torch.zeros(n, dtype=torch.float32).pin_memory()
        ckr.check(L.ckr_trace_closest_host(scene.handle, h_rays.data_ptr(), n, h_ids.data_ptr(), h_t.data_ptr(), 0),
                  "ckr_trace_closest_host")
        assert np.array_equal(h_ids.numpy().view(np.uint32), gid) and np.array_equal(h_t.numpy(), gt)
        h_rays.copy_(torch.from_numpy(rays))
        h_occ = torch.zeros(n, dtype=torch.uint8).pin_memory()
        ckr.check(L.ckr_trace_any_host(scene.handle, h_rays.data_ptr(), n, h_occ.data_ptr(), 0), "ckr_trace_any_host")
        assert np.array_equal(h_occ.numpy(), gocc)


def full_rays():
    tri = ckr.icosphere(8, 0.05, 6, 1)
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    primary = ckr.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    incoh = ckr.rays_incoherent(lo, hi, 7, 4194304, 0.05, 2.0)
    return tri, primary, incoh


@pytest.fixture(scope="module")
def full(torch_cuda):
    tri, primary, incoh = full_rays()
    scene = ckr.Scene(tri)
    return tri, primary, incoh, scene


def test_full_mesh_golden_sample(torch_cuda, full):
    tri, _, _, scene = full
    g = np.load(GOLD / "trace_full_sample.npz")
    gid, gt, occ = trace_device(torch_cuda, scene, closest_rays(g["rays"]))
    assert_parity(tri, g["rays"], gid, gt, g["ids"], g["t"], 1e-3)
    _, _, occ = trace_device(torch_cuda, scene, g["rays"])
    assert np.sum(occ != g["occluded"]) <= 2


def test_full_mesh_vs_oracle_subsample(torch_cuda, full):
    tri, primary, incoh, scene = full
    rays = np.concatenate([primary[::32], closest_rays(incoh[::32])])  # 262,144 rays
    gid, gt, _ = trace_device(torch_cuda, scene, rays)
    oid, ot = O.OracleBvh(tri).closest(rays)
    c = assert_parity(tri, rays, gid, gt, oid, ot, 1e-4)
    assert c["exact"] + c["tie"] + c["edge"] == len(rays)


def test_full_mesh_all_rays_properties(torch_cuda, full):
    """All 2^23 benchmark rays: closest/any consistency, determinism, hit validity."""
    tri, primary, incoh, scene = full
    rays = np.concatenate([primary, incoh])
    crays = closest_rays(rays)
    gid, gt, _ = trace_device(torch_cuda, scene, crays)
    gid2, gt2, _ = trace_device(torch_cuda, scene, crays)
    assert np.array_equal(gid, gid2) and np.array_equal(gt, gt2)
    _, _, occ = trace_device(torch_cuda, scene, rays)
    # any-hit(tmax) must equal [closest t < tmax] up to ties at tmax.
    expect = (gid != MISS) & (gt < rays[:, 7])
    diff = np.nonzero(occ.astype(bool) != expect)[0]
    assert len(diff) <= 1e-6 * len(rays) + 2, len(diff)
    # Every reported hit is a real FP64 hit of that triangle at (nearly) that distance.
    hits = np.nonzero(gid != MISS)[0]
    pick = np.random.default_rng(0).choice(hits, 4000, replace=False)
    for i in pick:
        t64, margin, _ = O.tri_intersect(tri[gid[i]], crays[i])
        if t64 < 1e19:
            assert abs(t64 - gt[i]) <= 1e-5 * max(1.0, t64)
        else:
            assert _boundary(tri, crays[i], int(gid[i]), float(gt[i])), (i, margin)
    # Primary rays: the sphere of radius ~1 at distance 3 covers the image centre.
    assert gid[2048 * 1024 + 1024] != MISS and gid[0] == MISS


def test_spheres_and_triangles(torch_cuda):
    tri = ckr.icosphere(2, 0.0, 1, 1) * np.float32(0.5)
    sph = np.array([[1.5, 0, 0, 0.5], [-1.5, 0, 0, 0.7], [0, 0, 0, 0.2], [0, 3, 0, 1.0]], dtype=np.float32)
    rays = np.concatenate([ckr.rays_pinhole([0, 0, 5], [0, 0, 0], [0, 1, 0], 60.0, 64, 64),
                           closest_rays(ckr.rays_incoherent([-2, -2, -2], [2, 2, 2], 3, 4096))])
    scene = ckr.Scene(tri, sph)
    gid, gt, occ = trace_device(torch_cuda, scene, rays)
    oid, ot = O.OracleBvh(tri).closest(rays)
    sid, st = O.spheres_closest(sph, rays)
    # Combined closest: sphere wins when strictly nearer (shade(), src/shader.cpp:355-357).
    ref_id = np.where(st < ot, sid | ckr.CKR_SPHERE_BIT, oid).astype(np.uint32)
    ref_t = np.minimum(st, ot)
    is_sph = (gid != MISS) & ((gid & ckr.CKR_SPHERE_BIT) != 0)
    both_sph = is_sph & (ref_id != MISS) & ((ref_id & ckr.CKR_SPHERE_BIT) != 0)
    assert np.array_equal(gid[both_sph], ref_id[both_sph])
    assert np.allclose(gt[both_sph], ref_t[both_sph], rtol=1e-6)
    mism = np.nonzero(gid != ref_id)[0]
    for i in mism:
        tie = abs(float(gt[i]) - ref_t[i]) <= 1e-5 * max(1.0, ref_t[i])
        g = int(gid[i])
        edge = (oid[i] != MISS and _boundary(tri, rays[i], int(oid[i]), float(ot[i]))) or \
               (g != MISS and not (g & ckr.CKR_SPHERE_BIT) and _boundary(tri, rays[i], g, float(gt[i])))
        assert tie or edge, i
    assert len(mism) <= 4


def test_degenerate_scenes(torch_cuda):
    rays = closest_rays(ckr.rays_incoherent([-1, -1, -1], [1, 1, 1], 5, 1000))
    # Empty scene: every ray misses.
    scene = ckr.Scene(None)
    gid, gt, occ = trace_device(torch_cuda, scene, rays)
    assert np.all(gid == MISS) and np.all(occ == 0) and np.all(gt == rays[:, 7])
    # Only degenerate / non-finite triangles.
    bad = np.array([[1e6] * 9, [0, 0, 0, 0, 0, 0, 0, 0, 0], [np.nan] * 9, [np.inf, 0, 0, 1, 0, 0, 0, 1, 0]],
                   dtype=np.float32)
    gid, _, occ = trace_device(torch_cuda, ckr.Scene(bad), rays)
    assert np.all(gid == MISS) and np.all(occ == 0)
    # A single triangle: the root is a leaf.
    one = np.array([[-1, -1, 0, 1, -1, 0, 0, 1, 0]], dtype=np.float32)
    r = closest_rays(np.array([[0, 0, 2, 0, 0, 0, -1, 1e30], [0.9, 0.9, 2, 0, 0, 0, -1, 1e30],
                               [0, 0, -2, 0, 0, 0, 1, 1e30], [0, 0, 2, 0, 0, 0, -1, 1.5]], dtype=np.float32))
    gid, gt, _ = trace_device(torch_cuda, ckr.Scene(one), r)
    assert list(gid) == [0, MISS, 0, 0] and abs(gt[0] - 2) < 1e-6 and abs(gt[2] - 2) < 1e-6
    _, _, occ = trace_device(torch_cuda, ckr.Scene(one), np.array([[0, 0, 2, 0, 0, 0, -1, 1.5],
                                                                   [0, 0, 2, 0, 0, 0, -1, 2.5]], dtype=np.float32))
    assert list(occ) == [0, 1]
