"""Save / load chakumrender_gb300.scene.SceneData as npz (test fixtures)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from chakumrender_gb300 import scene as S


def to_arrays(sd: S.SceneData, prefix: str) -> dict:
    mats = np.frombuffer(bytes(sd.materials)[: 64 * sd.nmat], dtype=np.uint8).copy()
    lights = np.frombuffer(bytes(sd.lights)[: 40 * sd.nlights], dtype=np.uint8).copy()
    cam = np.frombuffer(bytes(sd.camera), dtype=np.uint8).copy()
    return {f"{prefix}_tri9": sd.tri9, f"{prefix}_tri_mat": sd.tri_mat, f"{prefix}_sph4": sd.sph4,
            f"{prefix}_sph_mat": sd.sph_mat, f"{prefix}_mats": mats, f"{prefix}_lights": lights, f"{prefix}_cam": cam}


def from_arrays(g, prefix: str) -> S.SceneData:
    mb, lb = g[f"{prefix}_mats"].tobytes(), g[f"{prefix}_lights"].tobytes()
    mats = [S.Material.from_buffer_copy(mb[64 * i:64 * (i + 1)]) for i in range(len(mb) // 64)]
    lights = [S.Light.from_buffer_copy(lb[40 * i:40 * (i + 1)]) for i in range(len(lb) // 40)]
    cam = S.Camera.from_buffer_copy(g[f"{prefix}_cam"].tobytes())
    return S.SceneData(g[f"{prefix}_tri9"], g[f"{prefix}_tri_mat"], g[f"{prefix}_sph4"], g[f"{prefix}_sph_mat"], mats,
                       lights, cam)


def same_scene(a: S.SceneData, b: S.SceneData) -> bool:
    return (np.array_equal(a.tri9, b.tri9) and np.array_equal(a.tri_mat, b.tri_mat) and
            np.array_equal(a.sph4, b.sph4) and np.array_equal(a.sph_mat, b.sph_mat) and
            bytes(a.materials)[: 64 * a.nmat] == bytes(b.materials)[: 64 * b.nmat] and
            bytes(a.lights)[: 40 * a.nlights] == bytes(b.lights)[: 40 * b.nlights] and
            bytes(a.camera) == bytes(b.camera))


def srgb8(img: np.ndarray) -> np.ndarray:
    """The reference's display transform (src/main.cpp:27): clamp, gamma 1/2.2, int(x*255+.5)."""
    x = np.clip(np.nan_to_num(img, nan=0.0), 0, 1)
    return (x ** (1 / 2.2) * 255 + 0.5).astype(np.int32)


def block_agreement(img: np.ndarray, ref8: np.ndarray, block: int = 16):
    """Agreement of a linear render with an 8-bit reference image at the scale of
    16x16-pixel blocks (per-pixel 1-spp MIS noise averages out): both images go
    through the reference's display transform, back to linear, and are block-averaged;
    returns (mean, 99th percentile) of |a - b| / (b + 0.02) over blocks and channels."""
    def lin(v8):
        return (np.asarray(v8, np.float64) / 255.0) ** 2.2

    def blocks(a):
        h, w = a.shape[0] // block * block, a.shape[1] // block * block
        return a[:h, :w].reshape(h // block, block, w // block, block, 3).mean(axis=(1, 3))

    a, b = blocks(lin(srgb8(img))), blocks(lin(ref8))
    rel = np.abs(a - b) / (b + 0.02)
    return float(rel.mean()), float(np.quantile(rel, 0.99))


def rel_mse(a: np.ndarray, b: np.ndarray, eps: float = 1e-2) -> float:
    """mean((a - b)^2 / (b^2 + eps)) over pixels and channels (b is the reference)."""
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return float(np.mean((a - b) ** 2 / (b * b + eps)))


C.sizeof(S.Material)  # structures are defined
