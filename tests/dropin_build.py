"""Builds the C++ programs of the drop-in checks: the two main() programs of
INTEGRATION.md section 1 (extracted from the document, so the document is what is
compiled) and tests/cxx/dropin_queries.cpp, each against include/ and libckr.so."""
from __future__ import annotations

import re
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
LIBDIR = ROOT / "chakumrender_gb300"


def integration_programs() -> dict[str, str]:
    """The ```cpp blocks under the '### 1a.' and '### 1b.' headings."""
    text = (ROOT / "INTEGRATION.md").read_text()
    out = {}
    for key, head in (("dropin_main", "### 1a."), ("cabi_main", "### 1b.")):
        i = text.index(head)
        m = re.search(r"```cpp\n(.*?)```", text[i:], flags=re.S)
        assert m, f"no C++ block under {head}"
        out[key] = m.group(1)
    return out


def compile_program(src: Path, exe: Path) -> None:
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-fopenmp", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
           "-L", str(LIBDIR), "-lckr", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise AssertionError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build_all(tmp: Path) -> dict[str, Path]:
    exes = {}
    for name, code in integration_programs().items():
        src = tmp / f"{name}.cpp"
        src.write_text(code)
        exes[name] = tmp / name
        compile_program(src, exes[name])
    exes["queries"] = tmp / "dropin_queries"
    compile_program(ROOT / "tests" / "cxx" / "dropin_queries.cpp", exes["queries"])
    return exes


def read_pfm(path: Path) -> np.ndarray:
    """PFM as written by ckr_write_pfm: rows bottom to top on disk; returns top row first."""
    data = path.read_bytes()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"PF"
    w, h = map(int, parts[1].split())
    scale = float(parts[2])
    arr = np.frombuffer(parts[3][: w * h * 12], dtype="<f4" if scale < 0 else ">f4").reshape(h, w, 3)
    return arr[::-1].astype(np.float32)
