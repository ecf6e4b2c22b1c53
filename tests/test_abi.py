"""The C ABI: the library loads, exports every symbol include/ckr.h declares, and its
host-side argument checks work without a GPU."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np

from chakumrender_gb300 import ckr

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(ckr_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_exports_are_exactly_the_declared_entry_points():
    """Every ckr_* entry point the headers under include/ declare is exported, and
    nothing else is: no C++ internals, no template instantiations, no CUDA runtime."""
    syms = declared_symbols()
    assert len(syms) >= 14
    out = subprocess.run(["nm", "-D", "--defined-only", str(ckr.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    extra = sorted(exported - set(syms))
    assert not extra, extra[:10]
    L = ckr.lib()
    for s in syms:
        assert getattr(L, s) is not None


def test_status_strings():
    L = ckr.lib()
    buf = C.create_string_buffer(128)
    for code, word in [(0, "ok"), (-1, "invalid"), (-4, "stack"), (-5, "queue"), (-6, "iteration")]:
        assert L.ckr_status_string(code, buf, 128) == 0
        assert word in buf.value.decode()
    assert L.ckr_status_string(0, None, 0) == -1


def test_argument_checks_without_device():
    L = ckr.lib()
    h = C.c_void_p()
    # NULL output handle / NULL triangles with a count are rejected before any CUDA call.
    assert L.ckr_scene_create(None, 5, None, 0, None, None) == -1
    assert L.ckr_scene_create(None, 5, None, 0, None, C.byref(h)) == -1
    assert L.ckr_trace_closest(None, None, 0, None, None, None) == -1
    assert L.ckr_trace_stats(None, None, 0, None, None) == -1
    assert L.ckr_scene_destroy(None) == -1


def test_no_device_is_an_error_not_a_crash():
    import torch

    if torch.cuda.is_available():
        return
    tri = np.zeros((1, 9), dtype=np.float32)
    h = C.c_void_p()
    st = ckr.lib().ckr_scene_create(tri.ctypes.data, 1, None, 0, None, C.byref(h))
    assert st == -7  # CKR_ERR_NO_DEVICE
