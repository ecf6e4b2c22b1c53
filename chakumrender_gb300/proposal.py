"""ctypes wrapper of the learned light-selection proposal (ckr_proposal_*, include/ckr.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .ckr import _ptr, check, lib
from .scene import RenderCfg, RenderScene, Camera, _setup

P = C.c_void_p
U32 = C.c_uint32
NPARAMS = 18624


class ProposalCfg(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("lr", C.c_float), ("defensive", C.c_float), ("batch", U32), ("train", U32),
                ("minibatch", U32), ("max_steps", U32)]


def _sigs():
    L = _setup()
    if getattr(L, "_prop_sigs", False):
        return L
    for name, args in [("ckr_proposal_create", [P, P, C.POINTER(P)]), ("ckr_proposal_destroy", [P]),
                       ("ckr_proposal_set_training", [P, C.c_int]), ("ckr_proposal_get_params", [P, P]),
                       ("ckr_proposal_set_params", [P, P]), ("ckr_proposal_encoding", [P, P, P, P]),
                       ("ckr_proposal_infer", [P, P, U32, P, P]), ("ckr_proposal_train_step", [P, P, U32, P]),
                       ("ckr_proposal_status", [P, C.POINTER(U32), C.POINTER(C.c_float)]),
                       ("ckr_internal_proposal_gradients", [P, P, U32, P, C.POINTER(C.c_float)]),
                       ("ckr_render_learned", [P, P, P, P, P, P, P])]:
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L._prop_sigs = True
    return L


class Proposal:
    """Owns a ckr_proposal for a RenderScene."""

    def __init__(self, scene: RenderScene, seed=1, lr=1e-3, defensive=0.2, batch=65536, train=True,
                 minibatch=16384, max_steps=0):
        L = _sigs()
        self.scene = scene
        self._h = P()
        cfg = ProposalCfg(seed, lr, defensive, batch, 1 if train else 0, min(minibatch, batch), max_steps)
        check(L.ckr_proposal_create(scene.handle, C.byref(cfg), C.byref(self._h)), "ckr_proposal_create")

    @property
    def handle(self):
        return self._h.value

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().ckr_proposal_destroy(self._h)
            self._h = P()

    def set_training(self, on: bool):
        check(_sigs().ckr_proposal_set_training(self._h, int(on)), "set_training")

    def params(self) -> np.ndarray:
        out = np.empty(NPARAMS, np.float32)
        check(_sigs().ckr_proposal_get_params(self._h, _ptr(out)), "get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == NPARAMS
        check(_sigs().ckr_proposal_set_params(self._h, _ptr(p)), "set_params")

    def encoding(self):
        c = np.empty(3, np.float32)
        s, n = C.c_float(), U32()
        check(_sigs().ckr_proposal_encoding(self._h, _ptr(c), C.byref(s), C.byref(n)), "encoding")
        return c.astype(np.float64), float(s.value), int(n.value)

    def status(self):
        steps, loss = U32(), C.c_float()
        st = _sigs().ckr_proposal_status(self._h, C.byref(steps), C.byref(loss))
        return st, int(steps.value), float(loss.value)

    # Device-buffer forms (ints are device pointers).
    def infer(self, rec_dev: int, n: int, probs_dev: int, stream: int = 0):
        check(_sigs().ckr_proposal_infer(self._h, rec_dev, n, probs_dev, stream), "ckr_proposal_infer")

    def train_step(self, rec_dev: int, n: int, stream: int = 0):
        check(_sigs().ckr_proposal_train_step(self._h, rec_dev, n, stream), "ckr_proposal_train_step")

    def gradients(self, rec_dev: int, n: int):
        g = np.empty(NPARAMS, np.float32)
        loss = C.c_float()
        check(_sigs().ckr_internal_proposal_gradients(self._h, rec_dev, n, _ptr(g), C.byref(loss)), "gradients")
        return float(loss.value), g

    def render(self, cam: Camera, cfg: RenderCfg, rgb_dev: int, accum_dev: int | None = None, stream: int = 0):
        check(_sigs().ckr_render_learned(self.scene.handle, self._h, C.byref(cam), C.byref(cfg), rgb_dev,
                                         accum_dev, stream), "ckr_render_learned")
