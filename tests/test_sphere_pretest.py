"""The FP32 pre-test in front of the FP64 sphere test (hit_sphere, csrc/trace_device.cuh)
may only settle misses: wherever it reports a miss, the FP64 discriminant the reference's
Sphere::intersect computes (src/geometryPrimitives.cpp:12-27) must be negative too.  The
predicate is restated here in float32 and checked against float64 on random, grazing and
large-sphere cases.  No GPU."""
from __future__ import annotations

import numpy as np

F = np.float32


def pretest_miss(c, r, o, d):
    """The device predicate, float32 throughout (the device may fuse multiply-adds,
    which only rounds less)."""
    ox, oy, oz = (c[:, 0] - o[:, 0]), (c[:, 1] - o[:, 1]), (c[:, 2] - o[:, 2])
    b = ox * d[:, 0] + oy * d[:, 1] + oz * d[:, 2]
    oo = ox * ox + oy * oy + oz * oz
    dd = np.maximum(F(1), d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    m = np.maximum(np.abs(c).max(1), np.abs(o).max(1))
    with np.errstate(over="ignore", invalid="ignore"):
        return b * b - oo + r * r < F(-1e-5) * ((m * m + oo) * dd + b * b + r * r)


def fp64_det(c, r, o, d):
    op = c.astype(np.float64) - o.astype(np.float64)
    b = (op * d.astype(np.float64)).sum(1)
    return b * b - (op * op).sum(1) + r.astype(np.float64) ** 2


def unit(v):
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(F)


def test_pretest_never_rejects_a_hit():
    rng = np.random.default_rng(4)
    n = 400000
    cases = []
    # Small spheres near the origin (the box scene), rays from anywhere nearby.
    c = rng.uniform(-1, 1, (n, 3)).astype(F)
    r = rng.uniform(0.01, 0.5, n).astype(F)
    o = rng.uniform(-2, 2, (n, 3)).astype(F)
    cases.append((c, r, o, unit(rng.normal(size=(n, 3)))))
    # Grazing rays: aimed at a point on the silhouette, perturbed by 1e-7 .. 1e-3.
    d = unit(rng.normal(size=(n, 3)))
    side = unit(np.cross(d, rng.normal(size=(n, 3))))
    eps = 10 ** rng.uniform(-7, -3, n)
    target = c + side * (r * (1 + rng.choice([-1, 1], n) * eps))[:, None]
    o2 = (target - d * rng.uniform(0.5, 3, n)[:, None]).astype(F)
    cases.append((c, r, o2, unit(target - o2)))
    # The reference's 1e5-radius walls and far-off scenes.
    cw = (rng.normal(size=(n, 3)) * 1e5).astype(F)
    rw = (np.linalg.norm(cw, axis=1) * rng.uniform(0.999, 1.001, n)).astype(F)
    ow = rng.uniform(-50, 50, (n, 3)).astype(F)
    cases.append((cw, rw, ow, unit(rng.normal(size=(n, 3)))))
    co = (rng.uniform(-1, 1, (n, 3)) + 3e4).astype(F)
    cases.append((co, r, (co + rng.uniform(-3, 3, (n, 3))).astype(F), unit(rng.normal(size=(n, 3)))))
    # Directions of any length (the ABI does not require unit directions): |d| from
    # 1e-3 to 1e3 on the random and grazing cases, and rays whose length |d| = s puts
    # the reference's discriminant s^2 (op.u)^2 - |op|^2 + r^2 within 1e-7..1e-3 of 0.
    for c_, r_, o_, d_ in list(cases[:2]):
        s = (10 ** rng.uniform(-3, 3, n)).astype(F)[:, None]
        cases.append((c_, r_, o_, (d_ * s).astype(F)))
    op = (c - o).astype(np.float64)
    oo_ = (op * op).sum(1)
    s = 10 ** rng.uniform(0, 3, n)
    cos = np.sqrt(np.maximum(oo_ - r.astype(np.float64) ** 2, 0)) / (s * np.sqrt(oo_))
    ok = (oo_ > r.astype(np.float64) ** 2) & (cos < 1)
    perp = np.cross(op, rng.normal(size=(n, 3)))
    perp /= np.linalg.norm(perp, axis=1, keepdims=True)
    u = op / np.sqrt(oo_)[:, None] * cos[:, None] + perp * np.sqrt(np.maximum(1 - cos * cos, 0))[:, None]
    ds = u * (s * (1 + rng.choice([-1, 1], n) * 10 ** rng.uniform(-7, -3, n)))[:, None]
    cases.append((c[ok], r[ok], o[ok], ds[ok].astype(F)))
    culled = 0
    for c_, r_, o_, d_ in cases:
        miss = pretest_miss(c_, r_, o_, d_)
        det = fp64_det(c_, r_, o_, d_)
        assert not np.any(miss & (det >= 0)), np.nonzero(miss & (det >= 0))[0][:5]
        culled += int(miss.sum())
    # It must also do its job: most rays of the first case miss their sphere.
    assert culled > 0.5 * n


def leaving_miss(c, r, o, d):
    """The second device predicate (a ray leaving the sphere), float32 throughout."""
    ox, oy, oz = (c[:, 0] - o[:, 0]), (c[:, 1] - o[:, 1]), (c[:, 2] - o[:, 2])
    b = ox * d[:, 0] + oy * d[:, 1] + oz * d[:, 2]
    oo = ox * ox + oy * oy + oz * oz
    dd = np.maximum(F(1), d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    m = np.maximum(np.abs(c).max(1), np.abs(o).max(1))
    with np.errstate(over="ignore", invalid="ignore"):
        T = (m * m + oo) * dd + b * b + r * r
        det = b * b - oo + r * r
        t2u = (b + F(4e-6) * np.sqrt(T)) + np.sqrt(np.maximum(F(0), det + F(4e-6) * T))
        return t2u < F(5e-5)


def fp64_hits(c, r, o, d, tmin=0.0):
    """Sphere::intersect in FP64 (src/geometryPrimitives.cpp:12-27), root above
    max(1e-4, tmin): True where it reports a hit."""
    op = c.astype(np.float64) - o.astype(np.float64)
    b = (op * d.astype(np.float64)).sum(1)
    det = b * b - (op * op).sum(1) + r.astype(np.float64) ** 2
    s = np.sqrt(np.maximum(det, 0))
    eps = max(1e-4, tmin)
    return (det >= 0) & ((b - s > eps) | (b + s > eps))


def test_leaving_pretest_never_rejects_a_hit():
    """Rays from points on, just outside and just inside small and large spheres, in
    every direction (outward, grazing, inward), and rays from anywhere: wherever the
    second FP32 predicate reports a miss, the FP64 test reports one too; and at unit
    scale it settles most rays that leave a sphere from its surface (at large
    coordinates FP32 cannot resolve the 1e-4 margin and the FP64 test decides)."""
    rng = np.random.default_rng(9)
    n = 400000
    leaving = 0
    total_out = 0
    for scale, rad in ((1.0, (0.01, 0.5)), (1e3, (10.0, 300.0)), (1e-2, (1e-3, 5e-3))):
        c = (rng.uniform(-1, 1, (n, 3)) * scale).astype(F)
        r = rng.uniform(*rad, n).astype(F)
        nrm = unit(rng.normal(size=(n, 3)))
        # Origins on the surface, offset along the normal by -1e-3 .. 1e-3 of r.
        off = rng.uniform(-1e-3, 1e-3, n) * r
        o = (c + nrm * (r + off)[:, None]).astype(F)
        d = unit(rng.normal(size=(n, 3)))
        for d_ in (d, (d * (10 ** rng.uniform(-2, 2, n))[:, None]).astype(F)):
            miss = leaving_miss(c, r, o, d_)
            hit = fp64_hits(c, r, o, d_)
            assert not np.any(miss & hit), np.nonzero(miss & hit)[0][:5]
        if scale == 1.0:  # the box scene's scale: unit coordinates, radii 0.01 .. 0.5
            # Leaving from the surface or from just outside it, as bounce and shadow
            # rays do (their origins are offset along the normal); from just inside,
            # the FP64 test finds the exit point beyond 1e-4 and must decide.
            out = ((d * nrm).sum(1) > 0.3) & (off >= 0)
            total_out += int(out.sum())
            leaving += int((leaving_miss(c, r, o, d) & out).sum())
        # Rays from anywhere near the sphere.
        o2 = (c + rng.uniform(-3, 3, (n, 3)) * r[:, None]).astype(F)
        miss = leaving_miss(c, r, o2, d)
        assert not np.any(miss & fp64_hits(c, r, o2, d))
    assert leaving > 0.9 * total_out, (leaving, total_out)
