"""Generates the golden fixtures in tests/golden/ by running the REFERENCE renderer.

Needs oracle/_ref/libckr_ref.so (built by `make -C oracle ref REF=<checkout>` from the
reference's own sources) and libckr.so (for the deterministic input generators).  Run
from the repo root with CKR_REFERENCE naming the reference checkout:

    CKR_REFERENCE=<checkout> python tests/golden/make_golden.py

Fixtures:
  trace_small.npz        1280-triangle displaced icosphere; pinhole + incoherent rays;
                         the reference's BvhAccel::intersectT ids/t and shadow() booleans.
  trace_edges.npz        hand-built adversarial cases (shared edges, vertices, axis-aligned
                         and zero-component directions, grazing and in-plane rays, origins
                         on surfaces, degenerate triangles) with the reference's answers.
  trace_full_sample.npz  the 1,310,720-triangle mesh (digest only) and 4096 sampled rays of
                         the benchmark ray set with the reference's answers.
"""
from __future__ import annotations

import hashlib
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from chakumrender_gb300 import ckr  # noqa: E402
import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("CKR_REFERENCE", "")) if os.environ.get("CKR_REFERENCE") else None


def ray(o, d, tmax=1e30, tmin=0.0):
    return np.array([o[0], o[1], o[2], tmin, d[0], d[1], d[2], tmax], dtype=np.float32)


def normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return (v / np.linalg.norm(v)).astype(np.float32)


def edge_cases():
    rng = np.random.default_rng(11)
    ico = ckr.icosphere(2, 0.05, 6, 5)  # 320 triangles, shared edges/vertices
    ground = np.array([[-3, -1.5, -3, 3, -1.5, -3, 3, -1.5, 3],
                       [-3, -1.5, -3, 3, -1.5, 3, -3, -1.5, 3]], dtype=np.float32)
    degenerate = np.array([[1e6, 1e6, 1e6, 1e6, 1e6, 1e6, 1e6, 1e6, 1e6]], dtype=np.float32)
    sliver = np.array([[-2, 2, 0, 2, 2, 0, 0, 2.0001, 0]], dtype=np.float32)
    wall = np.array([[2.5, -2, -2, 2.5, 2, -2, 2.5, 2, 2]], dtype=np.float32)
    tri = np.concatenate([ico, ground, degenerate, sliver, wall])
    rays = []
    eye = np.array([0.3, 0.2, 4.0], dtype=np.float32)
    # Rays aimed at edge midpoints and vertices of the icosphere (shared features).
    for t in ico[rng.choice(len(ico), 64, replace=False)]:
        a, b, c = t[:3], t[3:6], t[6:]
        for p in (a, b, c, 0.5 * (a + b), 0.5 * (b + c), 0.5 * (c + a), (a + b + c) / 3):
            rays.append(ray(eye, normalize(p - eye)))
    # Axis-aligned directions from several origins (zero direction components).
    for o in ([0, 0, 3], [0.1, 0.2, -3], [3, 0.05, 0.02], [0, -3, 0.0], [0.2, 0.3, 0.4], [0, 0, 0]):
        for d in ([0, 0, -1], [0, 0, 1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0]):
            rays.append(ray(np.float32(o), np.float32(d)))
    # Rays in the ground plane and parallel to it (near-parallel rejection).
    for x in np.linspace(-2, 2, 9):
        rays.append(ray([x, -1.5, -4], [0, 0, 1]))
        rays.append(ray([x, -1.5 + 1e-4, -4], normalize([0, -1e-6, 1])))
        rays.append(ray([x, -1.0, -4], normalize([0, -1e-5, 1])))
        rays.append(ray([x, -1.0, -4], normalize([0, -0.2, 1])))
    # Grazing rays along the wall, rays hitting the sliver, rays toward the degenerate triangle.
    for y in np.linspace(-1.9, 1.9, 7):
        rays.append(ray([2.5, y, -3], [0, 0, 1]))
        rays.append(ray([0, 2.00005, -3], normalize([0.001 * y, 0, 1])))
        rays.append(ray([1e6 - 1, 1e6 - 1, 1e6 - 1], normalize([1, 1, 1])))
    # Origins on the surface (points inside triangles), shooting out and in.
    for t in ico[rng.choice(len(ico), 32, replace=False)]:
        a, b, c = t[:3].astype(np.float64), t[3:6].astype(np.float64), t[6:].astype(np.float64)
        p = ((a + b + c) / 3).astype(np.float32)
        n = normalize(np.cross(c - a, b - a))
        rays.append(ray(p, n))
        rays.append(ray(p, -n))
        rays.append(ray(p, normalize(rng.normal(size=3))))
    # Random rays through the whole setup, with shadow distances.
    for _ in range(256):
        o = rng.uniform(-3, 3, size=3).astype(np.float32)
        rays.append(ray(o, normalize(rng.normal(size=3)), tmax=float(rng.uniform(0.01, 5))))
    return tri, np.stack(rays)


def run_reference(tri, rays):
    rb = O.ReferenceBvh(tri)
    ids, t = rb.closest(rays)
    occ = rb.shadow(rays)
    return ids, t, occ


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def shading():
    """The reference's M_GGX, MaterialType::brdf / pdfEval (plain and LTC-approximate)
    and getLightFromMeshSource_Analytic on random inputs."""
    rng = np.random.default_rng(21)
    out = {}
    mg = np.stack([rng.uniform(0, 1.58, 256), rng.uniform(0, 1.1, 256)], 1).astype(np.float32)
    res = [O.m_ggx(float(t), float(a), reference=True) for t, a in mg]
    out.update(mggx_in=mg, mggx_M=np.stack([r[0] for r in res]), mggx_det=np.array([r[1] for r in res]),
               mggx_Minv=np.stack([r[2] for r in res]), mggx_amp=np.array([r[3] for r in res]))
    n = 2048
    nn = unit(rng, n)
    wo = unit(rng, n)
    wo[np.sum(wo * nn, 1) < 0] *= -1
    wi = unit(rng, n)
    wi[np.sum(wi * nn, 1) < 0] *= -1
    wo_ref = 2 * np.sum(nn * wo, 1, keepdims=True) * nn - wo
    mat = np.zeros(n, dtype=O.MATERIAL)
    mat["brdf"] = rng.integers(1, 5, n)
    mat["alpha"] = rng.uniform(0.05, 1, n)
    mat["alpha"][mat["brdf"] == 4] = rng.uniform(1, 200, int(np.sum(mat["brdf"] == 4)))
    mat["phong_exp"] = rng.uniform(1, 100, n)
    mat["spec"] = rng.uniform(0, 1, n)
    mat["int_ior"] = rng.uniform(1.1, 3, n)
    mat["ext_ior"] = 1.0
    b, p = O.brdf_batch(mat, nn, wo_ref, wo, wi, reference=True)
    mat_ltc = mat.copy()
    mat_ltc["brdf"] = 2
    mat_ltc["alpha"] = rng.uniform(0.05, 1, n)
    bl, _ = O.brdf_batch(mat_ltc, nn, wo_ref, wo, wi, use_ltc=True, reference=True)
    out.update(brdf_mat=mat, brdf_mat_ltc=mat_ltc, brdf_n=nn, brdf_wo_ref=wo_ref, brdf_wo=wo, brdf_wi=wi,
               brdf_out=b, brdf_pdf=p, brdf_out_ltc=bl)
    g = ckr.gbuffer(31, 1024)
    lt, lc = ckr.quad_lights(32, 8)
    m = np.zeros(len(g), dtype=O.MATERIAL)
    m["brdf"] = 2
    m["alpha"] = g[:, 3]
    m["spec"] = g[:, 11]
    f0 = g[:, 7].astype(np.float64)
    m["int_ior"] = (1 + np.sqrt(f0)) / (1 - np.sqrt(f0))
    m["ext_ior"] = 1.0
    x, nrm, v = g[:, 0:3].astype(np.float64), g[:, 4:7].astype(np.float64), g[:, 8:11].astype(np.float64)
    rgb = O.ltc_shade_batch(m, x, nrm, v, lt, lc, reference=True)
    out.update(ltc_gbuf=g, ltc_mat=m, ltc_x=x, ltc_n=nrm, ltc_v=v, ltc_tri=lt, ltc_rgb=lc, ltc_out=rgb)
    return out


def read_p3(path):
    t = Path(path).read_text().split()
    w, h = int(t[1]), int(t[2])
    return np.array(t[4:4 + w * h * 3], dtype=np.uint8).reshape(h, w, 3)


def reference_images():
    """The reference binary (oracle/_ref/a.out, default shader: shadeDirectOnly +
    getLightFromMeshSource_Analytic_MISCV, 1 spp at sub-pixel offset (0.34, 0.20))
    rendering the box scene and the reference's own scene0.xml; 8-bit P3 output."""
    import shutil
    import subprocess
    import tempfile

    exe = ROOT / "oracle" / "_ref" / "a.out"
    scenes = {"box": ROOT / "chakumrender_gb300" / "scenes" / "box.xml",
              "scene0": REFERENCE / "scene0.xml"}
    out = {}
    for name, xml in scenes.items():
        with tempfile.TemporaryDirectory() as d:
            shutil.copy(xml, Path(d) / "scene.xml")
            subprocess.run([str(exe), "scene.xml"], cwd=d, check=True, capture_output=True,
                           env={"OMP_NUM_THREADS": "8", "PATH": "/usr/bin:/bin"})
            out[name] = read_p3(Path(d) / "image.ppm")
    return out


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/libckr_ref.so is missing: run `make -C oracle ref REF=<checkout>` first")
    if REFERENCE is None or not (REFERENCE / "scene0.xml").exists():
        sys.exit("set CKR_REFERENCE to the reference checkout (its scene0.xml and scene1.xml are read)")
    np.savez_compressed(OUT / "ref_images.npz", **reference_images())
    print("reference images: written")
    # The reference's own scenes as parsed by the library's loader (which the CPU
    # tests check against the reference's prepareScene), for GPU tests on hosts
    # without the reference checkout.
    sys.path.insert(0, str(ROOT / "tests"))
    from chakumrender_gb300 import scene as S
    from scene_io import to_arrays

    arrays = {}
    for name in ("scene0", "scene1"):
        arrays.update(to_arrays(S.load_xml(str(REFERENCE / f"{name}.xml")), name))
    np.savez_compressed(OUT / "ref_scenes.npz", **arrays)
    print("reference scenes: written")
    np.savez_compressed(OUT / "shading.npz", **shading())
    print("shading: written")
    # Small mesh.
    tri = ckr.icosphere(3, 0.05, 6, 1)
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    r1 = ckr.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 48, 48)
    r2 = ckr.rays_incoherent(lo, hi, 7, 2048, 0.05, 2.0)
    rays = np.concatenate([r1, r2])
    ids, t, occ = run_reference(tri, rays)
    np.savez_compressed(OUT / "trace_small.npz", tri=tri, rays=rays, ids=ids, t=t, occluded=occ)
    print("trace_small:", len(tri), "tris", len(rays), "rays", "hit rate", float((ids != 0xFFFFFFFF).mean()))

    tri, rays = edge_cases()
    ids, t, occ = run_reference(tri, rays)
    np.savez_compressed(OUT / "trace_edges.npz", tri=tri, rays=rays, ids=ids, t=t, occluded=occ)
    print("trace_edges:", len(tri), "tris", len(rays), "rays", "hit rate", float((ids != 0xFFFFFFFF).mean()))

    tri = ckr.icosphere(8, 0.05, 6, 1)
    digest = hashlib.sha256(tri.tobytes()).hexdigest()
    lo, hi = tri.reshape(-1, 3).min(0), tri.reshape(-1, 3).max(0)
    r1 = ckr.rays_pinhole([0, 0, 3], [0, 0, 0], [0, 1, 0], 40.0, 2048, 2048)
    r2 = ckr.rays_incoherent(lo, hi, 7, 4194304, 0.05, 2.0)
    pick = np.random.default_rng(3).choice(len(r1), 2048, replace=False)
    rays = np.concatenate([r1[pick], r2[pick]])
    ids, t, occ = run_reference(tri, rays)
    np.savez_compressed(OUT / "trace_full_sample.npz", mesh_sha256=np.array(digest), ray_index=pick,
                        rays=rays, ids=ids, t=t, occluded=occ)
    print("trace_full_sample:", digest[:16], len(rays), "rays")


if __name__ == "__main__":
    main()
