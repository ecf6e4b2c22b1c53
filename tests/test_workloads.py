"""Synthetic workload generators: determinism, sizes and distributions."""
from __future__ import annotations

import numpy as np

from chakumrender_gb300 import ckr


def test_icosphere_sizes_and_radius():
    for sub in range(0, 5):
        tri = ckr.icosphere(sub, 0.05, 6, 1)
        assert tri.shape == (20 * 4 ** sub, 9)
        r = np.linalg.norm(tri.reshape(-1, 3), axis=1)
        assert r.min() >= 0.95 - 1e-6 and r.max() <= 1.05 + 1e-6


def test_icosphere_is_watertight_and_deterministic():
    a = ckr.icosphere(3, 0.05, 6, 7)
    b = ckr.icosphere(3, 0.05, 6, 7)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, ckr.icosphere(3, 0.05, 6, 8))
    # Every edge is shared by exactly two triangles with bit-identical endpoints.
    v = a.reshape(-1, 3, 3)
    edges = {}
    for t in v:
        for i in range(3):
            p, q = tuple(t[i]), tuple(t[(i + 1) % 3])
            key = (min(p, q), max(p, q))
            edges[key] = edges.get(key, 0) + 1
    assert set(edges.values()) == {2}


def test_rays():
    r = ckr.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 64, 32)
    assert r.shape == (2048, 8)
    d = r[:, 4:7].astype(np.float64)
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
    assert np.all(r[:, 3] == 0) and np.all(r[:, 7] == np.float32(1e30))
    # Top-left pixel looks up and left; pixel centres are symmetric about the axis.
    assert d[0, 0] < 0 and d[0, 1] > 0
    assert np.allclose(d[:, 0].reshape(32, 64), -d[:, 0].reshape(32, 64)[:, ::-1], atol=1e-6)
    lo, hi = np.array([-1, -2, -3]), np.array([1, 2, 3])
    q = ckr.rays_incoherent(lo, hi, 7, 20000, 0.05, 2.0)
    assert np.all(q[:, :3] >= lo) and np.all(q[:, :3] <= hi)
    dq = q[:, 4:7].astype(np.float64)
    assert np.allclose(np.linalg.norm(dq, axis=1), 1.0, atol=1e-6)
    assert np.all(np.abs(dq.mean(0)) < 0.02)
    assert np.allclose(dq.T @ dq / len(dq), np.eye(3) / 3, atol=0.02)
    assert q[:, 7].min() >= 0.05 and q[:, 7].max() <= 2.0
    assert np.array_equal(q, ckr.rays_incoherent(lo, hi, 7, 20000, 0.05, 2.0))


def test_rng_stream():
    xs = np.array([ckr.rng_uniform(1, 5, c) for c in range(4000)])
    assert xs.min() >= 0 and xs.max() < 1
    assert abs(xs.mean() - 0.5) < 0.02
    assert np.all(xs * 16777216 == np.floor(xs * 16777216))  # 24-bit values


def test_oracle_generator_is_byte_identical():
    """The oracle's C restatement of the workload (used by the CPU timing of the
    reference traversal, which must not load the library) gives the same bytes as
    ckr_workload_*."""
    import oracle as O

    for sub, seed in ((0, 1), (3, 7), (5, 1)):
        assert np.array_equal(ckr.icosphere(sub, 0.05, 6, seed).view(np.uint32),
                              O.icosphere(sub, 0.05, 6, seed).view(np.uint32))
    a = ckr.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 96, 64)
    b = O.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 96, 64)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    lo, hi = np.array([-1.05, -1.04, -1.03], np.float32), np.array([1.02, 1.05, 1.01], np.float32)
    a = ckr.rays_incoherent(lo, hi, 7, 50000, 0.05, 2.0)
    b = O.rays_incoherent(lo, hi, 7, 50000, 0.05, 2.0)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    a = ckr.rays_incoherent(lo, hi, 7, 50000)
    b = O.rays_incoherent(lo, hi, 7, 50000)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
