"""ctypes structures and wrappers for full scenes and rendering (include/ckr.h)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .ckr import BuildParams, Scene, _ptr, check, lib

P = C.c_void_p
U32 = C.c_uint32
F3 = C.c_float * 3

SHADER_DIRECT_MISCV = 0
SHADER_DIRECT_MIS = 1
SHADER_PATH = 2
SHADER_PATH_NEE = 3
SHADER_DIRECT_CV = 4
SHADER_EXPLICIT = 5
LIGHT_MESH, LIGHT_TRI, LIGHT_SPHERE, LIGHT_POINT = 0, 1, 2, 3
SCENES = Path(__file__).resolve().parent / "scenes"


class Material(C.Structure):
    _fields_ = [("brdf", C.c_int32), ("light_type", C.c_int32), ("alpha", C.c_float), ("phong_exp", C.c_float),
                ("spec", C.c_float), ("int_ior", C.c_float), ("ext_ior", C.c_float), ("reflectance", C.c_float),
                ("color", F3), ("radiance", F3), ("pad", C.c_float * 2)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("first", U32), ("count", U32), ("pos", F3), ("power", F3),
                ("pad", C.c_float)]


class EnvLight(C.Structure):
    _fields_ = [("rgb", P), ("width", U32), ("height", U32), ("axis", U32), ("color", F3), ("intensity", C.c_float),
                ("n_samples", U32)]


class SceneDesc(C.Structure):
    _fields_ = [("tri9", P), ("tri_material", P), ("ntri", U32), ("sph4", P), ("sph_material", P), ("nsph", U32),
                ("materials", P), ("nmaterials", U32), ("lights", P), ("nlights", U32), ("build", BuildParams),
                ("env", C.POINTER(EnvLight))]


class Camera(C.Structure):
    _fields_ = [("pos", F3), ("dir", F3), ("cx", F3), ("cy", F3), ("width", U32), ("height", U32)]


class RenderCfg(C.Structure):
    _fields_ = [("shader", U32), ("spp", U32), ("max_depth", U32), ("n_light_samples", U32),
                ("n_brdf_samples", U32), ("rr_prob", C.c_float), ("seed", C.c_uint64), ("flags", U32),
                ("reserved", U32)]


assert C.sizeof(Material) == 64 and C.sizeof(Light) == 40 and C.sizeof(RenderCfg) == 40
assert C.sizeof(Camera) == 56


def _setup():
    L = lib()
    if getattr(L, "_scene_sigs", False):
        return L
    for name, args in [("ckr_scene_create_ex", [P, C.POINTER(P)]), ("ckr_render", [P, P, P, P, P, P]),
                       ("ckr_render_host", [P, P, P, P, P]), ("ckr_write_ppm", [C.c_char_p, P, U32, U32]),
                       ("ckr_xml_load", [C.c_char_p, C.POINTER(P)]), ("ckr_xml_get", [P, P, P]),
                       ("ckr_xml_free", [P]),
                       ("ckr_render_stats", [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int])]:
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L._scene_sigs = True
    return L


def render_cfg(shader=SHADER_PATH, spp=16, max_depth=4, n_light=1, n_brdf=1, rr_prob=0.3, seed=1) -> RenderCfg:
    return RenderCfg(shader, spp, max_depth, n_light, n_brdf, rr_prob, seed, 0, 0)


class SceneData:
    """Host-side scene description (arrays kept alive for the descriptor)."""

    def __init__(self, tri9, tri_mat, sph4, sph_mat, materials, lights, camera: Camera | None = None, env=None):
        self.tri9 = np.ascontiguousarray(tri9, np.float32).reshape(-1, 9)
        self.tri_mat = np.ascontiguousarray(tri_mat, np.uint32)
        self.sph4 = np.ascontiguousarray(sph4, np.float32).reshape(-1, 4)
        self.sph_mat = np.ascontiguousarray(sph_mat, np.uint32)
        if isinstance(materials, C.Array):  # already a ctypes array (large scenes)
            self.materials, self.nmat = materials, len(materials)
        else:
            self.materials = (Material * max(1, len(materials)))(*materials)
            self.nmat = len(materials)
        if isinstance(lights, C.Array):
            self.lights, self.nlights = lights, len(lights)
        else:
            self.lights = (Light * max(1, len(lights)))(*lights)
            self.nlights = len(lights)
        self.camera = camera
        self.env = None
        if env is not None:
            self.set_env(*env) if isinstance(env, tuple) else self.set_env(**env)

    def set_env(self, image, axis: int = 1, color=(1.0, 1.0, 1.0), intensity: float = 1.0, n_samples: int = 0):
        """Environment light (ckr_env_light): image (h, w, 3) equirectangular about `axis`."""
        self.env_image = np.ascontiguousarray(image, np.float32).reshape(image.shape[0], image.shape[1], 3)
        h, w = self.env_image.shape[:2]
        self.env = EnvLight(_ptr(self.env_image), w, h, axis, F3(*color), intensity, n_samples)

    def desc(self, max_leaf: int = 0) -> SceneDesc:
        return SceneDesc(_ptr(self.tri9) if len(self.tri9) else None, _ptr(self.tri_mat) if len(self.tri9) else None,
                         len(self.tri9), _ptr(self.sph4) if len(self.sph4) else None,
                         _ptr(self.sph_mat) if len(self.sph4) else None, len(self.sph4),
                         C.addressof(self.materials), self.nmat, C.addressof(self.lights), self.nlights,
                         BuildParams(max_leaf, 0, 0), C.pointer(self.env) if self.env is not None else None)


def load_xml(path) -> SceneData:
    """initSceneParser + prepare* through the library's XML loader."""
    L = _setup()
    h = P()
    check(L.ckr_xml_load(str(path).encode(), C.byref(h)), f"ckr_xml_load({path})")
    try:
        d, cam = SceneDesc(), Camera()
        check(L.ckr_xml_get(h, C.byref(d), C.byref(cam)), "ckr_xml_get")

        def arr(ptr, n, dtype, k):
            if n == 0 or not ptr:
                return np.zeros((0, k) if k > 1 else 0, dtype)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dtype))),
                                         shape=(n * k,)).copy().reshape((n, k) if k > 1 else n)

        mats = [Material.from_buffer_copy(C.string_at(d.materials + i * 64, 64)) for i in range(d.nmaterials)]
        lights = [Light.from_buffer_copy(C.string_at(d.lights + i * 40, 40)) for i in range(d.nlights)]
        return SceneData(arr(d.tri9, d.ntri, np.float32, 9), arr(d.tri_material, d.ntri, np.uint32, 1),
                         arr(d.sph4, d.nsph, np.float32, 4), arr(d.sph_material, d.nsph, np.uint32, 1), mats, lights,
                         cam)
    finally:
        L.ckr_xml_free(h)


class RenderScene(Scene):
    """A ckr_scene with shading data (ckr_scene_create_ex)."""

    def __init__(self, data: SceneData, max_leaf: int = 0):
        L = _setup()
        self._h = P()
        self.data = data
        d = data.desc(max_leaf)
        check(L.ckr_scene_create_ex(C.byref(d), C.byref(self._h)), "ckr_scene_create_ex")

    def render_host(self, cam: Camera, cfg: RenderCfg, stream: int = 0) -> np.ndarray:
        out = np.empty((cam.height, cam.width, 3), np.float32)
        check(_setup().ckr_render_host(self._h, C.byref(cam), C.byref(cfg), _ptr(out), stream), "ckr_render_host")
        return out

    def render(self, cam: Camera, cfg: RenderCfg, rgb_dev: int, accum_dev: int | None = None, stream: int = 0):
        check(_setup().ckr_render(self._h, C.byref(cam), C.byref(cfg), rgb_dev, accum_dev, stream), "ckr_render")

    def ray_stats(self, reset: bool = True):
        a, b = C.c_uint64(), C.c_uint64()
        check(_setup().ckr_render_stats(self._h, C.byref(a), C.byref(b), int(reset)), "ckr_render_stats")
        return a.value, b.value


def write_ppm(path, rgb: np.ndarray) -> None:
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w = rgb.shape[:2]
    check(_setup().ckr_write_ppm(str(path).encode(), _ptr(rgb), w, h), "ckr_write_ppm")


class ManylightSpec(C.Structure):
    _fields_ = [("subdiv", U32), ("octaves", U32), ("noise_amp", C.c_float), ("mesh_seed", C.c_uint64),
                ("rough_seed", C.c_uint64), ("emit_seed", C.c_uint64), ("alpha_lo", C.c_float),
                ("alpha_hi", C.c_float), ("mesh_spec", C.c_float), ("mesh_albedo", C.c_float),
                ("room_albedo", C.c_float), ("floor_y", C.c_float), ("nemit", U32), ("nclusters", U32),
                ("emit_side", C.c_float), ("radiance_lo", C.c_float), ("radiance_hi", C.c_float),
                ("cam_pos", F3), ("cam_target", F3), ("fov_deg", C.c_float), ("width", U32), ("height", U32)]


def manylight_spec(subdiv=8, nemit=4096, nclusters=64, width=1920, height=1080, **kw) -> ManylightSpec:
    """The many-light scene: the 1,310,720-triangle displaced icosphere (GGX, roughness
    uniform per triangle in [0.1, 0.8], seed 3) in a 10^3 diffuse room with 4,096
    emissive triangles on its ceiling and walls (radiance log-uniform in [0.5, 50])
    grouped into 64 clusters."""
    s = ManylightSpec(subdiv=subdiv, octaves=6, noise_amp=0.05, mesh_seed=1, rough_seed=3, emit_seed=5,
                      alpha_lo=0.1, alpha_hi=0.8, mesh_spec=1.0, mesh_albedo=0.9, room_albedo=0.7, floor_y=-1.2,
                      nemit=nemit, nclusters=nclusters, emit_side=0.12, radiance_lo=0.5, radiance_hi=50.0,
                      cam_pos=F3(0.0, 0.6, 3.4), cam_target=F3(0.0, 0.0, 0.0), fov_deg=45.0, width=width,
                      height=height)
    for k, v in kw.items():
        setattr(s, k, F3(*v) if k in ("cam_pos", "cam_target") else v)
    return s


def manylight_scene(spec: ManylightSpec | None = None) -> SceneData:
    L = lib()
    if not getattr(L, "_ml_sig", False):
        L.ckr_workload_manylight.argtypes = [P, P, P, P, P, P, P]
        L.ckr_workload_manylight.restype = C.c_int
        L._ml_sig = True
    spec = spec or manylight_spec()
    counts = (U32 * 3)()
    check(L.ckr_workload_manylight(C.byref(spec), None, None, None, None, None, counts), "manylight size")
    ntri, nmat, nl = counts
    tri = np.empty((ntri, 9), np.float32)
    tri_mat = np.empty(ntri, np.uint32)
    mats = (Material * nmat)()
    lights = (Light * nl)()
    cam = Camera()
    check(L.ckr_workload_manylight(C.byref(spec), _ptr(tri), _ptr(tri_mat), C.addressof(mats), C.addressof(lights),
                                   C.byref(cam), counts), "manylight")
    return SceneData(tri, tri_mat, np.zeros((0, 4), np.float32), np.zeros(0, np.uint32), mats, lights, cam)
