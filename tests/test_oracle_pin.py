"""Pins the FP64 oracle to the reference renderer.

The golden fixtures in tests/golden/ hold the reference's own answers
(BvhAccel::intersectT ids and t, shadow() booleans), produced by
tests/golden/make_golden.py from oracle/_ref (the reference compiled from its
sources).  The oracle must reproduce them bit for bit.  Where oracle/_ref is
present (the development container), the oracle is also compared against the
live reference on fresh inputs.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import oracle as O
from chakumrender_gb300 import ckr

GOLD = Path(__file__).resolve().parent / "golden"


def closest_rays(rays):
    r = rays.copy()
    r[:, 7] = 1e30
    return r


@pytest.mark.parametrize("name", ["trace_small", "trace_edges"])
def test_oracle_matches_reference_golden(name):
    g = np.load(GOLD / f"{name}.npz")
    ob = O.OracleBvh(g["tri"])
    ids, t = ob.closest(g["rays"])
    assert np.array_equal(ids, g["ids"])
    assert np.array_equal(t, g["t"])
    assert np.array_equal(ob.shadow(g["rays"]), g["occluded"])


def test_oracle_matches_reference_golden_full_mesh():
    g = np.load(GOLD / "trace_full_sample.npz")
    tri = ckr.icosphere(8, 0.05, 6, 1)
    import hashlib

    assert hashlib.sha256(tri.tobytes()).hexdigest() == str(g["mesh_sha256"])
    ob = O.OracleBvh(tri)
    ids, t = ob.closest(g["rays"])
    assert np.array_equal(ids, g["ids"])
    assert np.array_equal(t, g["t"])
    assert np.array_equal(ob.shadow(g["rays"]), g["occluded"])


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not built here")
@pytest.mark.parametrize("seed", [2, 9])
def test_oracle_matches_live_reference(seed):
    tri = ckr.icosphere(4, 0.1, 3, seed)
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    rays = np.concatenate([ckr.rays_pinhole([0.2, 0.1, 2.5], [0, 0, 0], [0, 1, 0], 50.0, 40, 30),
                           ckr.rays_incoherent(lo, hi, seed, 3000, 0.05, 1.5)])
    ob, rb = O.OracleBvh(tri), O.ReferenceBvh(tri)
    a, b = ob.closest(rays), rb.closest(rays)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(ob.shadow(rays), rb.shadow(rays))
