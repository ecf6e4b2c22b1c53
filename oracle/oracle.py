"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

liboracle.so is the FP64 C restatement of the reference (oracle/*.c); libckr_ref.so is
the reference renderer itself compiled from its own sources (oracle/_ref/, present
only where the reference sources were available to build it).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_SO = HERE / "_ref" / "libckr_ref.so"
LTC_TABLE = HERE.parent / "chakumrender_gb300" / "data" / "ltc_ggx.bin"

# orc_material / the reference's MaterialType fields (brdf: 0 NONE, 1 CLASSIC_PHONG,
# 2 GGX, 3 BECKMANN, 4 PHONG, 5 GGXAPPROX).
MATERIAL = np.dtype([("brdf", "<i4"), ("pad", "<i4"), ("alpha", "<f8"), ("phong_exp", "<f8"), ("spec", "<f8"),
                     ("int_ior", "<f8"), ("ext_ior", "<f8")])

P = C.c_void_p
U32 = C.c_uint32
_orc = None
_ref = None


def _sig(lib, name, args, res=C.c_int):
    f = getattr(lib, name)
    f.argtypes = args
    f.restype = res


def orc() -> C.CDLL:
    global _orc
    if _orc is None:
        L = C.CDLL(str(ORACLE_SO))
        _sig(L, "orc_bvh_build", [P, U32], P)
        _sig(L, "orc_bvh_free", [P], None)
        _sig(L, "orc_bvh_node_count", [P], U32)
        _sig(L, "orc_trace_closest", [P, P, U32, P, P, P, P, C.c_int], None)
        _sig(L, "orc_trace_shadow", [P, P, U32, P, C.c_int], None)
        _sig(L, "orc_tri_intersect", [P, P, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_double)
        _sig(L, "orc_spheres_closest", [P, U32, P, U32, P, P], None)
        _sig(L, "orc_tri_edge_distance", [P, P, C.POINTER(C.c_double)], C.c_double)
        _sig(L, "orc_ltc_load", [C.c_char_p])
        _sig(L, "orc_m_ggx", [C.c_float, C.c_float, P, P, P, P], None)
        _sig(L, "orc_brdf_batch", [P, U32, P, P, P, P, C.c_int, P, P], None)
        _sig(L, "orc_ltc_shade_batch", [P, U32, P, P, P, P, P, U32, P, C.c_int], None)
        _sig(L, "orc_sample_dir", [C.c_int, P, P, C.c_double, C.c_double, C.c_double, P], None)
        _sig(L, "orc_workload_icosphere", [U32, C.c_float, U32, C.c_uint64, P, U32, C.POINTER(U32)])
        _sig(L, "orc_workload_rays_pinhole", [P, P, P, C.c_float, U32, U32, C.c_float, P])
        _sig(L, "orc_workload_rays_incoherent", [P, P, C.c_uint64, U32, C.c_float, C.c_float, P])
        _sig(L, "orc_ltc_mc", [P, U32, P, P, P, P, P, U32, U32, C.c_uint64, P, P, C.c_int], None)
        _sig(L, "orc_mlp_forward", [P, P, U32, P, C.c_double, U32, P], None)
        _sig(L, "orc_mlp_loss_grad", [P, P, U32, P, C.c_double, U32, P, P], C.c_int)
        _sig(L, "orc_mlp_adam", [P, P, P, P, U32, U32, C.c_double, C.c_double, C.c_double, C.c_double], None)
        _sig(L, "orc_mlp_features", [P, P, C.c_double, P], None)
        if L.orc_ltc_load(str(LTC_TABLE).encode()) != 0:
            raise RuntimeError(f"cannot load {LTC_TABLE}")
        _orc = L
    return _orc


def ref_available() -> bool:
    return REF_SO.exists()


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        L = C.CDLL(str(REF_SO))
        _sig(L, "ref_trace_build", [P, U32])
        _sig(L, "ref_trace_closest", [P, U32, P, P, C.c_int], None)
        _sig(L, "ref_trace_shadow", [P, U32, P, C.c_int], None)
        _sig(L, "ref_read_image", [C.c_char_p, P, U32, P, P])
        _sig(L, "ref_write_image", [C.c_char_p, P, U32, U32])
        _ref = L
    return _ref


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def icosphere(subdiv: int = 8, noise_amp: float = 0.05, octaves: int = 6, seed: int = 1) -> np.ndarray:
    """The displaced icosphere of the traversal workload, made without the library."""
    n = C.c_uint32(0)
    if orc().orc_workload_icosphere(subdiv, noise_amp, octaves, seed, None, 0, C.byref(n)) != 0:
        raise ValueError("icosphere size")
    out = np.empty((n.value, 9), dtype=np.float32)
    if orc().orc_workload_icosphere(subdiv, noise_amp, octaves, seed, _p(out), n.value, C.byref(n)) != 0:
        raise RuntimeError("orc_workload_icosphere failed")
    return out


def rays_pinhole(eye, target, up, vfov_deg: float, width: int, height: int, tmax: float = 1e30) -> np.ndarray:
    e, t, u = (np.ascontiguousarray(x, dtype=np.float32) for x in (eye, target, up))
    out = np.empty((width * height, 8), dtype=np.float32)
    if orc().orc_workload_rays_pinhole(_p(e), _p(t), _p(u), vfov_deg, width, height, tmax, _p(out)) != 0:
        raise ValueError("orc_workload_rays_pinhole: invalid camera")
    return out


def rays_incoherent(lo, hi, seed: int, n: int, tmax_lo: float = 1e30, tmax_hi: float = 1e30) -> np.ndarray:
    lo, hi = (np.ascontiguousarray(x, dtype=np.float32) for x in (lo, hi))
    out = np.empty((n, 8), dtype=np.float32)
    if orc().orc_workload_rays_incoherent(_p(lo), _p(hi), seed, n, tmax_lo, tmax_hi, _p(out)) != 0:
        raise ValueError("orc_workload_rays_incoherent")
    return out


class OracleBvh:
    """The reference's midpoint BVH and intersectT, restated in FP64 C."""

    def __init__(self, tri9: np.ndarray):
        self.tri9 = np.ascontiguousarray(tri9, dtype=np.float32).reshape(-1, 9)
        self._h = orc().orc_bvh_build(_p(self.tri9), len(self.tri9))
        if not self._h:
            raise MemoryError("orc_bvh_build failed")

    def node_count(self) -> int:
        return orc().orc_bvh_node_count(self._h)

    def closest(self, rays: np.ndarray, threads: int = 0, counts: bool = False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = len(rays)
        ids = np.empty(n, dtype=np.uint32)
        t = np.empty(n, dtype=np.float64)
        nv = np.empty(n, dtype=np.uint32) if counts else None
        nt = np.empty(n, dtype=np.uint32) if counts else None
        orc().orc_trace_closest(self._h, _p(rays), n, _p(ids), _p(t), _p(nv) if counts else None,
                                _p(nt) if counts else None, threads)
        return (ids, t, nv, nt) if counts else (ids, t)

    def shadow(self, rays: np.ndarray, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        occ = np.empty(len(rays), dtype=np.uint8)
        orc().orc_trace_shadow(self._h, _p(rays), len(rays), _p(occ), threads)
        return occ

    def __del__(self):
        try:
            if self._h:
                orc().orc_bvh_free(self._h)
                self._h = None
        except Exception:
            pass


def spheres_closest(sph4: np.ndarray, rays: np.ndarray):
    """Nearest sphere per ray by the reference's Sphere::intersect (FP64)."""
    sph = np.ascontiguousarray(sph4, dtype=np.float32).reshape(-1, 4)
    rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    ids = np.empty(len(rays), dtype=np.uint32)
    t = np.empty(len(rays), dtype=np.float64)
    orc().orc_spheres_closest(_p(sph), len(sph), _p(rays), len(rays), _p(ids), _p(t))
    return ids, t


def tri_intersect(tri9_row: np.ndarray, ray8: np.ndarray):
    """Reference Triangle::intersect on one triangle: (t, barycentric margin, |d.n|)."""
    tri = np.ascontiguousarray(tri9_row, dtype=np.float32).reshape(9)
    ray = np.ascontiguousarray(ray8, dtype=np.float32).reshape(8)
    m, dn = C.c_double(), C.c_double()
    t = orc().orc_tri_intersect(_p(tri), _p(ray), C.byref(m), C.byref(dn))
    return t, m.value, dn.value


def tri_edge_distance(tri9_row: np.ndarray, ray8: np.ndarray):
    """(signed distance from the plane hit point to the triangle boundary, plane t)."""
    tri = np.ascontiguousarray(tri9_row, dtype=np.float32).reshape(9)
    ray = np.ascontiguousarray(ray8, dtype=np.float32).reshape(8)
    tp = C.c_double()
    d = orc().orc_tri_edge_distance(_p(tri), _p(ray), C.byref(tp))
    return d, tp.value


class ReferenceBvh:
    """The unmodified reference (BvhAccel::intersectT, shadow()) via oracle/_ref/libckr_ref.so.

    The reference keeps its scene in process globals, so one instance at a time."""

    def __init__(self, tri9: np.ndarray):
        self.tri9 = np.ascontiguousarray(tri9, dtype=np.float32).reshape(-1, 9)
        if ref().ref_trace_build(_p(self.tri9), len(self.tri9)) != 0:
            raise RuntimeError("ref_trace_build failed")

    def closest(self, rays: np.ndarray, threads: int = 0):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        ids = np.empty(len(rays), dtype=np.uint32)
        t = np.empty(len(rays), dtype=np.float64)
        ref().ref_trace_closest(_p(rays), len(rays), _p(ids), _p(t), threads)
        return ids, t

    def shadow(self, rays: np.ndarray, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        occ = np.empty(len(rays), dtype=np.uint8)
        ref().ref_trace_shadow(_p(rays), len(rays), _p(occ), threads)
        return occ


# ---- materials, samplers, LTC -----------------------------------------------------------
def _d3(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3)


def m_ggx(theta: float, alpha: float, reference: bool = False):
    """M_GGX: (M row-major 9, det(M) of the lower theta entry, Minv 9, amplitude)."""
    M, Mi = np.empty(9), np.empty(9)
    det, amp = C.c_double(), C.c_double()
    lib = _ref_shading_sigs() if reference else orc()
    lib.ref_m_ggx(theta, alpha, _p(M), C.byref(det), _p(Mi), C.byref(amp)) if reference else \
        lib.orc_m_ggx(theta, alpha, _p(M), C.byref(det), _p(Mi), C.byref(amp))
    return M, det.value, Mi, amp.value


def brdf_batch(mat, n, wo_ref, wo, wi, use_ltc=False, reference=False):
    """MaterialType::brdf and ::pdfEval per row."""
    mat = np.ascontiguousarray(mat, dtype=MATERIAL)
    n, wo_ref, wo, wi = _d3(n), _d3(wo_ref), _d3(wo), _d3(wi)
    out, pdf = np.empty(len(mat)), np.empty(len(mat))
    f = _ref_shading_sigs().ref_brdf_batch if reference else orc().orc_brdf_batch
    f(_p(mat), len(mat), _p(n), _p(wo_ref), _p(wo), _p(wi), int(use_ltc), _p(out), _p(pdf))
    return out, pdf


def ltc_shade_batch(mat, x, n, v, light_tri9, light_rgb, reference=False, threads=0):
    """getLightFromMeshSource_Analytic per shading point (v = view direction = -r.d)."""
    mat = np.ascontiguousarray(mat, dtype=MATERIAL)
    x, n, v = _d3(x), _d3(n), _d3(v)
    lt = np.ascontiguousarray(light_tri9, dtype=np.float32).reshape(-1, 9)
    lc = np.ascontiguousarray(light_rgb, dtype=np.float32).reshape(-1, 3)
    out = np.empty((len(mat), 3))
    f = _ref_shading_sigs().ref_ltc_shade_batch if reference else orc().orc_ltc_shade_batch
    f(_p(mat), len(mat), _p(x), _p(n), _p(v), _p(lt), _p(lc), len(lt), _p(out), threads)
    return out


def ltc_mc(mat, x, n, v, light_tri9, light_rgb, spp: int, seed: int, pixel_index=None, threads: int = 0):
    """FP64 Monte Carlo of the integral the LTC shading approximates (see orc_render.inc)."""
    mat = np.ascontiguousarray(mat, dtype=MATERIAL)
    x, n, v = _d3(x), _d3(n), _d3(v)
    lt = np.ascontiguousarray(light_tri9, dtype=np.float32).reshape(-1, 9)
    lc = np.ascontiguousarray(light_rgb, dtype=np.float32).reshape(-1, 3)
    idx = None if pixel_index is None else np.ascontiguousarray(pixel_index, dtype=np.uint32)
    out = np.empty((len(mat), 3))
    orc().orc_ltc_mc(_p(mat), len(mat), _p(x), _p(n), _p(v), _p(lt), _p(lc), len(lt), spp, seed,
                     None if idx is None else _p(idx), _p(out), threads)
    return out


MLP_NPARAMS = 64 * 96 + 3 * (64 * 64 + 64)


def mlp_features(rec12, centre, scale) -> np.ndarray:
    rec = np.ascontiguousarray(rec12, dtype=np.float32).reshape(-1, 12)
    c = np.ascontiguousarray(centre, dtype=np.float64)
    out = np.empty((len(rec), 96))
    for i in range(len(rec)):
        orc().orc_mlp_features(rec[i].ctypes.data, _p(c), scale, out[i].ctypes.data)
    return out


def mlp_forward(params, rec12, centre, scale, nclusters) -> np.ndarray:
    """The light-selection network in FP64: n x 64 probabilities (see orc_mlp.c)."""
    prm = np.ascontiguousarray(params, dtype=np.float64)
    rec = np.ascontiguousarray(rec12, dtype=np.float32).reshape(-1, 12)
    c = np.ascontiguousarray(centre, dtype=np.float64)
    out = np.empty((len(rec), 64))
    orc().orc_mlp_forward(_p(prm), _p(rec), len(rec), _p(c), scale, nclusters, _p(out))
    return out


def mlp_loss_grad(params, rec12, centre, scale, nclusters):
    """(loss, gradient) of the training objective over the records; (0, zeros) if all weights are 0."""
    prm = np.ascontiguousarray(params, dtype=np.float64)
    rec = np.ascontiguousarray(rec12, dtype=np.float32).reshape(-1, 12)
    c = np.ascontiguousarray(centre, dtype=np.float64)
    g = np.empty(MLP_NPARAMS)
    loss = C.c_double(0)
    orc().orc_mlp_loss_grad(_p(prm), _p(rec), len(rec), _p(c), scale, nclusters, _p(g), C.byref(loss))
    return loss.value, g


def mlp_adam(params, m, v, grad, step, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    """In place on float64 arrays params, m, v."""
    for a in (params, m, v):
        assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    g = np.ascontiguousarray(grad, dtype=np.float64)
    orc().orc_mlp_adam(_p(params), _p(m), _p(v), _p(g), len(params), step, lr, beta1, beta2, eps)


def sample_dir(kind: int, n, w, param: float, e1: float, e2: float) -> np.ndarray:
    """One direction sample of the reference samplers from uniforms (see orc_shading.c)."""
    n = np.ascontiguousarray(n, dtype=np.float64).reshape(3)
    w = np.ascontiguousarray(w if w is not None else n, dtype=np.float64).reshape(3)
    out = np.empty(3)
    orc().orc_sample_dir(kind, _p(n), _p(w), param, e1, e2, _p(out))
    return out


def _ref_shading_sigs():
    L = ref()
    if not hasattr(L, "_shading"):
        _sig(L, "ref_m_ggx", [C.c_float, C.c_float, P, P, P, P], None)
        _sig(L, "ref_brdf_batch", [P, U32, P, P, P, P, C.c_int, P, P], None)
        _sig(L, "ref_ltc_shade_batch", [P, U32, P, P, P, P, P, U32, P, C.c_int], None)
        L._shading = True
    return L


def render(scene_data, cam, cfg, threads: int = 0) -> np.ndarray:
    """The reference's shaders restated in FP64 with the library's RNG streams:
    (height, width, 3) linear RGB, top row first (chakumrender_gb300.scene structs)."""
    L = orc()
    if not hasattr(L, "_render"):
        _sig(L, "orc_render", [P, P, P, P, C.c_int], None)
        L._render = True
    d = scene_data.desc()
    out = np.empty((cam.height, cam.width, 3), np.float64)
    L.orc_render(C.byref(d), C.byref(cam), C.byref(cfg), _p(out), threads)
    return out


def env_eval(env, dirs):
    """The oracle's environment lookup: (n, 4) radiance rgb + luminance, and the
    luminance integral A.  `env` is a chakumrender_gb300.scene.EnvLight."""
    L = orc()
    if not hasattr(L, "_env"):
        _sig(L, "orc_env_eval", [P, P, U32, P, P], None)
        _sig(L, "orc_env_sample", [P, P, U32, P], None)
        L._env = True
    dirs = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    out = np.empty((len(dirs), 4), np.float64)
    area = C.c_double()
    L.orc_env_eval(C.byref(env), _p(dirs), len(dirs), _p(out), C.byref(area))
    return out, area.value


def env_sample(env, u):
    """Directions drawn by the oracle's environment sampler from uniforms u (n, 3)."""
    env_eval(env, np.zeros((0, 3)))  # signatures
    u = np.ascontiguousarray(u, np.float64).reshape(-1, 3)
    out = np.empty((len(u), 3), np.float64)
    orc().orc_env_sample(C.byref(env), _p(u), len(u), _p(out))
    return out


def ref_env(image, axis, color, intensity, dirs, nsamples=0):
    """The reference's EnvSource: getRadiance per direction, normalizationArea, and
    the first nsamples of its importance-sampled directions."""
    L = ref()
    if not hasattr(L, "_env"):
        _sig(L, "ref_env", [P, U32, U32, U32, P, C.c_double, P, U32, P, P, P, U32])
        L._env = True
    img = np.ascontiguousarray(image, np.float64)
    h, w = img.shape[:2]
    dirs = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    col = np.ascontiguousarray(color, np.float64)
    rgb = np.empty((len(dirs), 3), np.float64)
    area = C.c_double()
    smp = np.empty((max(nsamples, 1), 3), np.float64)
    L.ref_env(_p(img), w, h, axis, _p(col), intensity, _p(dirs), len(dirs), _p(rgb), C.byref(area), _p(smp), nsamples)
    return rgb, area.value, smp[:nsamples]
