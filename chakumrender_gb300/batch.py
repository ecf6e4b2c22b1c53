"""ctypes wrapper of batched rendering (ckr_batch_*, include/ckr.h) and the batch
workload: box-scene jobs with random sphere BRDFs, camera yaw, resolution, spp and
depth."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from .ckr import check, lib
from .scene import Camera, Material, RenderScene, SceneData, _setup

P = C.c_void_p
U32 = C.c_uint32


class Job(C.Structure):
    _fields_ = [("cam", Camera), ("spp", U32), ("max_depth", U32), ("seed", C.c_uint64), ("material_set", U32),
                ("reserved", U32), ("rgb", P)]


class BatchTuning(C.Structure):
    _fields_ = [("block", U32), ("wave", U32), ("ms", C.c_float), ("candidates", U32), ("mode", U32)]


def _sigs():
    L = _setup()
    if getattr(L, "_batch_sigs", False):
        return L
    for name, args in [("ckr_batch_create", [P, U32, C.c_float, U32, P, U32, P, U32, P, C.POINTER(P)]),
                       ("ckr_batch_render", [P, P]), ("ckr_batch_render_sequential", [P, P]),
                       ("ckr_batch_get_tuning", [P, P]), ("ckr_batch_get_stats", [P, P, P]),
                       ("ckr_batch_destroy", [P])]:
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L._batch_sigs = True
    return L


class Batch:
    """Owns a ckr_batch (jobs, material tables, the captured graph)."""

    def __init__(self, scene: RenderScene, jobs, materials=None, shader=2, rr_prob=0.3, n_light=1, tuning=None):
        L = _sigs()
        self.scene = scene
        self.jobs = (Job * len(jobs))(*jobs)
        self.nsets = 0 if materials is None else len(materials) // scene.data.nmat
        self.materials = materials
        self._h = P()
        tp = C.byref(tuning) if tuning is not None else None
        mats = C.addressof(materials) if materials is not None else None
        check(L.ckr_batch_create(scene.handle, shader, rr_prob, n_light, mats, self.nsets, C.addressof(self.jobs),
                                 len(jobs), tp, C.byref(self._h)), "ckr_batch_create")

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().ckr_batch_destroy(self._h)
            self._h = P()

    def render(self, stream: int = 0):
        check(_sigs().ckr_batch_render(self._h, stream), "ckr_batch_render")

    def render_sequential(self, stream: int = 0):
        check(_sigs().ckr_batch_render_sequential(self._h, stream), "ckr_batch_render_sequential")

    def tuning(self) -> BatchTuning:
        t = BatchTuning()
        check(_sigs().ckr_batch_get_tuning(self._h, C.byref(t)), "ckr_batch_get_tuning")
        return t

    def stats(self):
        paths, launches = C.c_uint64(), U32()
        check(_sigs().ckr_batch_get_stats(self._h, C.byref(paths), C.byref(launches)), "ckr_batch_get_stats")
        return paths.value, launches.value


def _rot_y(v, c, s):
    return np.array([c * v[0] + s * v[2], v[1], -s * v[0] + c * v[2]])


def box_jobs(sd: SceneData, njobs=64, seed=4, sizes=(256, 512, 768, 1024), spps=(4, 16, 64), depths=(3, 6)):
    """The batch workload over the box scene: per job a material set with the two
    spheres' BRDF drawn from GGX / Beckmann / microfacet Phong and roughness uniform
    in [0.05, 0.9] (Phong exponent 2 / r^2 - 2), the camera turned about the box's
    vertical axis by a yaw uniform in [-30, 30] degrees, resolution, spp and depth
    uniform over the given choices.  Returns (job parameters, material sets as one
    ctypes array); the jobs' rgb pointers are filled in by the caller."""
    rng = np.random.default_rng(seed)
    base = [Material.from_buffer_copy(sd.materials[i]) for i in range(sd.nmat)]
    sph_mats = sorted({int(m) for m in sd.sph_mat[:2]})  # the two spheres; the third is the reference's dummy
    sets = []
    params = []
    cam0 = sd.camera
    centre = np.array([0.5, 0.0, 0.5])
    for j in range(njobs):
        mats = [Material.from_buffer_copy(m) for m in base]
        for k in sph_mats:
            brdf = int(rng.choice([2, 3, 4]))
            r = float(rng.uniform(0.05, 0.9))
            mats[k].brdf = brdf
            mats[k].alpha = r if brdf != 4 else 2.0 / (r * r) - 2.0
        sets.extend(mats)
        yaw = math.radians(float(rng.uniform(-30, 30)))
        c, s = math.cos(yaw), math.sin(yaw)
        size = int(rng.choice(sizes))
        cam = Camera()
        pos = centre + _rot_y(np.array(cam0.pos, float) - centre, c, s)
        for k, v in enumerate(pos):
            cam.pos[k] = v
        for name in ("dir", "cx", "cy"):
            v = _rot_y(np.array(getattr(cam0, name), float), c, s)
            for k in range(3):
                getattr(cam, name)[k] = v[k]
        cam.width = cam.height = size
        params.append(dict(cam=cam, spp=int(rng.choice(spps)), max_depth=int(rng.choice(depths)),
                           seed=1000 + j, material_set=j))
    return params, (Material * len(sets))(*sets)
