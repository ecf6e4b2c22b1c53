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
        _ref = L
    return _ref


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


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
