"""ctypes binding of libckr.so (the C ABI declared in include/ckr.h).

This is a thin convenience layer for Python callers (tests, bench.py); the C ABI is
the product boundary.  Host arrays are numpy; device buffers are raw pointers (for
example torch CUDA tensors' data_ptr()).  There is no fallback: if libckr.so is
missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libckr.so"

CKR_OK = 0
CKR_MISS = 0xFFFFFFFF
CKR_SPHERE_BIT = 0x80000000


CKR_ERR_INVALID_ARGUMENT, CKR_ERR_PARSE, CKR_ERR_IO, CKR_ERR_TOO_LARGE = -1, -8, -9, -10


class CkrError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {status_string(status)} ({status})")


class BuildParams(C.Structure):
    _fields_ = [("max_leaf_size", C.c_uint32), ("sah_bins", C.c_uint32), ("threads", C.c_uint32)]


class SceneInfo(C.Structure):
    _fields_ = [("ntri", C.c_uint32), ("nsph", C.c_uint32), ("nnodes", C.c_uint32), ("nleaves", C.c_uint32),
                ("max_depth", C.c_uint32), ("nnodes_binary", C.c_uint32), ("device_bytes", C.c_uint64),
                ("build_ms", C.c_double)]


_lib: C.CDLL | None = None
P = C.c_void_p
U32 = C.c_uint32
F32 = C.c_float


def _sig(lib, name, args, res=C.c_int):
    f = getattr(lib, name)
    f.argtypes = args
    f.restype = res
    return f


def lib() -> C.CDLL:
    """Loads libckr.so (built by chakumrender_gb300.build); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise FileNotFoundError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
    L = C.CDLL(str(LIB_PATH))
    _sig(L, "ckr_status_string", [C.c_int, C.c_char_p, C.c_size_t])
    _sig(L, "ckr_scene_create", [P, U32, P, U32, C.POINTER(BuildParams), C.POINTER(P)])
    _sig(L, "ckr_scene_destroy", [P])
    _sig(L, "ckr_scene_get_info", [P, C.POINTER(SceneInfo)])
    _sig(L, "ckr_scene_check", [P, P])
    _sig(L, "ckr_trace_closest", [P, P, U32, P, P, P])
    _sig(L, "ckr_trace_any", [P, P, U32, P, P])
    _sig(L, "ckr_trace_closest_host", [P, P, U32, P, P, P])
    _sig(L, "ckr_trace_any_host", [P, P, U32, P, P])
    _sig(L, "ckr_trace_stats", [P, P, U32, C.POINTER(C.c_double), C.POINTER(C.c_double)])
    _sig(L, "ckr_obj_load", [C.c_char_p, P, U32, C.POINTER(U32)])
    _sig(L, "ckr_read_ppm_p6", [C.c_char_p, P, U32, C.POINTER(U32), C.POINTER(U32)])
    _sig(L, "ckr_write_ppm_p6", [C.c_char_p, P, U32, U32])
    _sig(L, "ckr_write_pfm", [C.c_char_p, P, U32, U32])
    _sig(L, "ckr_workload_icosphere", [U32, F32, U32, C.c_uint64, P, U32, C.POINTER(U32)])
    _sig(L, "ckr_workload_rays_pinhole", [P, P, P, F32, U32, U32, F32, P])
    _sig(L, "ckr_workload_rays_incoherent", [P, P, C.c_uint64, U32, F32, F32, P])
    _sig(L, "ckr_rng_uniform", [C.c_uint64, C.c_uint64, U32], F32)
    _sig(L, "ckr_ltc_init", [C.c_char_p])
    _sig(L, "ckr_ltc_shade", [P, U32, P, P, U32, P, P])
    _sig(L, "ckr_ltc_mc", [P, U32, P, P, U32, U32, C.c_uint64, C.c_int, P, P])
    _sig(L, "ckr_workload_gbuffer", [C.c_uint64, U32, P])
    _sig(L, "ckr_workload_quad_lights", [C.c_uint64, U32, F32, F32, F32, P, P])
    _lib = L
    return L


def gbuffer(seed: int, npx: int) -> np.ndarray:
    out = np.empty((npx, 12), dtype=np.float32)
    check(lib().ckr_workload_gbuffer(seed, npx, _ptr(out)), "gbuffer")
    return out


def quad_lights(seed: int, nquads: int = 8, side_lo: float = 0.2, side_hi: float = 1.0, radiance: float = 5.0):
    tri = np.empty((2 * nquads, 9), dtype=np.float32)
    rgb = np.empty((2 * nquads, 3), dtype=np.float32)
    check(lib().ckr_workload_quad_lights(seed, nquads, side_lo, side_hi, radiance, _ptr(tri), _ptr(rgb)),
          "quad_lights")
    return tri, rgb


def ltc_shade(gbuf_dev: int, npx: int, light_tri_dev: int, light_rgb_dev: int, nlight: int, rgb_dev: int,
              stream: int = 0) -> None:
    check(lib().ckr_ltc_shade(gbuf_dev, npx, light_tri_dev, light_rgb_dev, nlight, rgb_dev, stream), "ckr_ltc_shade")


def ltc_mc(gbuf_dev: int, npx: int, light_tri_dev: int, light_rgb_dev: int, nlight: int, spp: int, seed: int,
           fresnel: bool, rgb_dev: int, stream: int = 0) -> None:
    """Monte Carlo reference of the LTC integral (device buffers; rgb: npx x 3 doubles)."""
    check(lib().ckr_ltc_mc(gbuf_dev, npx, light_tri_dev, light_rgb_dev, nlight, spp, seed, int(fresnel), rgb_dev,
                           stream), "ckr_ltc_mc")


def status_string(status: int) -> str:
    buf = C.create_string_buffer(512)
    if _lib is None:
        return "libckr not loaded"
    _lib.ckr_status_string(status, buf, 512)
    return buf.value.decode()


def check(status: int, what: str) -> None:
    if status != CKR_OK:
        raise CkrError(status, what)


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _f3(v) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(3))


# ---- synthetic workloads ---------------------------------------------------------
def load_obj(path) -> np.ndarray:
    """Triangles of a Wavefront OBJ file as an (n, 9) float32 array (ckr_obj_load)."""
    L = lib()
    n = U32(0)
    p = str(path).encode()
    check(L.ckr_obj_load(p, None, 0, C.byref(n)), "ckr_obj_load size")
    out = np.empty((n.value, 9), dtype=np.float32)
    if n.value:
        check(L.ckr_obj_load(p, _ptr(out), n.value, C.byref(n)), "ckr_obj_load")
    return out


def read_ppm_p6(path) -> np.ndarray:
    """(h, w, 3) float32 image of a binary P6 file (ckr_read_ppm_p6)."""
    L = lib()
    w, h = U32(0), U32(0)
    p = str(path).encode()
    check(L.ckr_read_ppm_p6(p, None, 0, C.byref(w), C.byref(h)), "ckr_read_ppm_p6 size")
    out = np.empty((h.value, w.value, 3), dtype=np.float32)
    check(L.ckr_read_ppm_p6(p, _ptr(out), w.value * h.value, C.byref(w), C.byref(h)), "ckr_read_ppm_p6")
    return out


def write_ppm_p6(path, rgb: np.ndarray) -> None:
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    check(lib().ckr_write_ppm_p6(str(path).encode(), _ptr(rgb), rgb.shape[1], rgb.shape[0]), "ckr_write_ppm_p6")


def write_pfm(path, rgb: np.ndarray) -> None:
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    check(lib().ckr_write_pfm(str(path).encode(), _ptr(rgb), rgb.shape[1], rgb.shape[0]), "ckr_write_pfm")


def icosphere(subdiv: int = 8, noise_amp: float = 0.05, octaves: int = 6, seed: int = 1) -> np.ndarray:
    L = lib()
    n = U32(0)
    check(L.ckr_workload_icosphere(subdiv, noise_amp, octaves, seed, None, 0, C.byref(n)), "icosphere size")
    out = np.empty((n.value, 9), dtype=np.float32)
    check(L.ckr_workload_icosphere(subdiv, noise_amp, octaves, seed, _ptr(out), n.value, C.byref(n)), "icosphere")
    return out


def rays_pinhole(eye, target, up, vfov_deg: float, width: int, height: int, tmax: float = 1e30) -> np.ndarray:
    out = np.empty((width * height, 8), dtype=np.float32)
    e, t, u = _f3(eye), _f3(target), _f3(up)
    check(lib().ckr_workload_rays_pinhole(_ptr(e), _ptr(t), _ptr(u), vfov_deg, width, height, tmax, _ptr(out)),
          "rays_pinhole")
    return out


def rays_incoherent(lo, hi, seed: int, n: int, tmax_lo: float = 1e30, tmax_hi: float = 1e30) -> np.ndarray:
    out = np.empty((n, 8), dtype=np.float32)
    a, b = _f3(lo), _f3(hi)
    check(lib().ckr_workload_rays_incoherent(_ptr(a), _ptr(b), seed, n, tmax_lo, tmax_hi, _ptr(out)),
          "rays_incoherent")
    return out


def rng_uniform(seed: int, index: int, counter: int) -> float:
    return float(lib().ckr_rng_uniform(seed, index, counter))


# ---- scene + traversal -------------------------------------------------------------
class Scene:
    """Owns a ckr_scene handle (BVH + geometry in device memory)."""

    def __init__(self, tri9: np.ndarray | None, spheres: np.ndarray | None = None,
                 max_leaf_size: int = 0, sah_bins: int = 0, threads: int = 0):
        L = lib()
        self._h = P()
        tri = np.ascontiguousarray(tri9, dtype=np.float32).reshape(-1, 9) if tri9 is not None else None
        sph = np.ascontiguousarray(spheres, dtype=np.float32).reshape(-1, 4) if spheres is not None else None
        params = BuildParams(max_leaf_size, sah_bins, threads)
        st = L.ckr_scene_create(_ptr(tri) if tri is not None and len(tri) else None,
                                len(tri) if tri is not None else 0,
                                _ptr(sph) if sph is not None and len(sph) else None,
                                len(sph) if sph is not None else 0, C.byref(params), C.byref(self._h))
        check(st, "ckr_scene_create")

    @property
    def handle(self) -> int:
        return self._h.value

    def info(self) -> SceneInfo:
        inf = SceneInfo()
        check(lib().ckr_scene_get_info(self._h, C.byref(inf)), "ckr_scene_get_info")
        return inf

    def check_device(self, stream: int = 0) -> int:
        return lib().ckr_scene_check(self._h, stream)

    def trace_closest_host(self, rays: np.ndarray, stream: int = 0):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = len(rays)
        ids = np.empty(n, dtype=np.uint32)
        t = np.empty(n, dtype=np.float32)
        check(lib().ckr_trace_closest_host(self._h, _ptr(rays), n, _ptr(ids), _ptr(t), stream),
              "ckr_trace_closest_host")
        return ids, t

    def trace_any_host(self, rays: np.ndarray, stream: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        occ = np.empty(len(rays), dtype=np.uint8)
        check(lib().ckr_trace_any_host(self._h, _ptr(rays), len(rays), _ptr(occ), stream), "ckr_trace_any_host")
        return occ

    def trace_closest(self, rays_dev: int, n: int, hit_id_dev: int, hit_t_dev: int, stream: int = 0) -> None:
        check(lib().ckr_trace_closest(self._h, rays_dev, n, hit_id_dev, hit_t_dev, stream), "ckr_trace_closest")

    def trace_any(self, rays_dev: int, n: int, occluded_dev: int, stream: int = 0) -> None:
        check(lib().ckr_trace_any(self._h, rays_dev, n, occluded_dev, stream), "ckr_trace_any")

    def stats(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        b, t = C.c_double(), C.c_double()
        check(lib().ckr_trace_stats(self._h, _ptr(rays), len(rays), C.byref(b), C.byref(t)), "ckr_trace_stats")
        return b.value, t.value

    def close(self) -> None:
        if self._h and self._h.value:
            lib().ckr_scene_destroy(self._h)
            self._h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
