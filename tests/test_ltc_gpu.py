"""GPU parity of ckr_ltc_shade (LTC polygon-light shading) against the reference's own
answers (golden fixture) and the FP64 oracle; full-size (1024^2 G-buffer) properties."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from chakumrender_gb300 import ckr
from test_ltc_host import host_replay, ltc_errors, oracle_ltc

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
REL_TOL = 1e-4  # per pixel, relative to the pixel's magnitude (floored at 1% of the image mean)


def shade_gpu(torch, g, lt, lc):
    dg = torch.from_numpy(np.ascontiguousarray(g, np.float32)).cuda()
    dt = torch.from_numpy(np.ascontiguousarray(lt, np.float32)).cuda()
    dc = torch.from_numpy(np.ascontiguousarray(lc, np.float32)).cuda()
    out = torch.empty((len(g), 3), dtype=torch.float32, device="cuda")
    ckr.ltc_shade(dg.data_ptr(), len(g), dt.data_ptr(), dc.data_ptr(), len(lt), out.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
    return out.cpu().numpy()


def test_golden_reference(torch_cuda):
    g = np.load(GOLD / "shading.npz")
    got = shade_gpu(torch_cuda, g["ltc_gbuf"], g["ltc_tri"], g["ltc_rgb"])
    err = ltc_errors(got, g["ltc_out"])
    assert err.max() <= REL_TOL, np.sort(err)[-10:]


def test_vs_oracle_and_host_replay(torch_cuda):
    g = ckr.gbuffer(77, 65536)
    lt, lc = ckr.quad_lights(78, 8)
    got = shade_gpu(torch_cuda, g, lt, lc)
    assert ltc_errors(got, oracle_ltc(g, lt, lc)).max() <= REL_TOL
    # Same FP32 code on the host: differences only from FMA contraction and libm.
    assert ltc_errors(got, host_replay(g, lt, lc)).max() <= REL_TOL


def test_full_size_properties(torch_cuda):
    """1024^2 G-buffer, 8 quads: finite, non-negative, linear in the emitted radiance,
    additive over emitters, deterministic; a 16k-pixel sample against the oracle."""
    g = ckr.gbuffer(2, 1024 * 1024)
    lt, lc = ckr.quad_lights(3, 8)
    a = shade_gpu(torch_cuda, g, lt, lc)
    assert np.all(np.isfinite(a)) and a.min() >= 0 and a.mean() > 0
    assert np.array_equal(a, shade_gpu(torch_cuda, g, lt, lc))
    # Doubling the radiance doubles the result exactly (power-of-two scaling).
    assert np.array_equal(2 * a, shade_gpu(torch_cuda, g, lt, 2 * lc))
    # Additivity: first four quads + last four quads.
    b = shade_gpu(torch_cuda, g, lt[:8], lc[:8]) + shade_gpu(torch_cuda, g, lt[8:], lc[8:])
    assert np.max(np.abs(a - b) / np.maximum(a, 1e-3 * a.mean())) < 1e-5
    pick = np.random.default_rng(0).choice(len(g), 16384, replace=False)
    assert ltc_errors(a[pick], oracle_ltc(g[pick], lt, lc)).max() <= REL_TOL


def test_many_emitters_fill_the_warp_queues(torch_cuda):
    """96 quads (192 emitter triangles): a warp of 32 pixels meets far more triangles
    across the horizon than its 256-entry queue holds, so lanes also clip in place
    once the queue is full; both routes agree with the oracle, and repeated launches
    give the same bits."""
    g = ckr.gbuffer(91, 4096)
    lt, lc = ckr.quad_lights(92, 96, 0.5, 3.0)
    got = shade_gpu(torch_cuda, g, lt, lc)
    assert np.all(np.isfinite(got)) and got.min() >= 0 and got.mean() > 0
    assert np.array_equal(got, shade_gpu(torch_cuda, g, lt, lc))
    assert ltc_errors(got, oracle_ltc(g, lt, lc)).max() <= REL_TOL
