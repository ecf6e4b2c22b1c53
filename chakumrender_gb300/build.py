"""Builds libckr.so in-tree: CUDA sources with nvcc for sm_103a, host C++ with g++.

Objects go to chakumrender_gb300/_build/, the library to chakumrender_gb300/libckr.so.
Translation units compile in parallel; an object is rebuilt when its source or any
header under csrc/ or include/ is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libckr.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden", "-fvisibility-inlines-hidden",
              "-Wall"]
# Exports: the ckr_* entry points the headers under include/ declare, nothing else.
VERSION_SCRIPT = PKG / "csrc" / "exports.map"


def _nvcc() -> str:
    p = CUDA_HOME / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")) + [VERSION_SCRIPT]
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile_cmd(src: Path, obj: Path) -> list[str]:
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    if src.suffix == ".cu":
        return [_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden,-fvisibility-inlines-hidden", "-Xptxas", "-warn-spills",
                *inc, "-c", str(src), "-o", str(obj)]
    return ["g++", *HOST_FLAGS, *inc, "-I", str(CUDA_HOME / "include"), "-c", str(src), "-o", str(obj)]


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    hdr_t = _headers_mtime()
    todo = []
    for s in srcs:
        obj = BUILD / (s.name + ".o")
        if not obj.exists() or obj.stat().st_mtime < max(s.stat().st_mtime, hdr_t):
            todo.append((s, obj))

    def run(job):
        s, obj = job
        cmd = _compile_cmd(s, obj)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout.strip() or r.stderr.strip()):
            print(r.stdout + r.stderr, file=sys.stderr)
        return s.name

    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for name in ex.map(run, todo):
            if verbose:
                print(f"[build] compiled {name}", file=sys.stderr)
    objs = [str(BUILD / (s.name + ".o")) for s in srcs]
    newest = max(Path(o).stat().st_mtime for o in objs)
    if todo or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *objs, "-lpthread",
               "-Xlinker", f"--version-script={VERSION_SCRIPT}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
        if verbose:
            print(f"[build] linked {LIB}", file=sys.stderr)
    return LIB


def reference_checkout() -> Path | None:
    """The reference checkout named by the CKR_REFERENCE environment variable, if it
    holds the reference's sources (there is no default location)."""
    ref = os.environ.get("CKR_REFERENCE")
    if ref and (Path(ref) / "src" / "bvhAccel.cpp").exists():
        return Path(ref)
    return None


def build_oracle(verbose: bool = False) -> None:
    """Builds oracle/liboracle.so, and oracle/_ref/ when CKR_REFERENCE names the
    reference's sources."""
    odir = ROOT / "oracle"
    targets = ["all"]
    ref = reference_checkout()
    extra = []
    if ref is not None:
        targets.append("ref")
        extra = [f"REF={ref}"]
    cmd = ["make", "-s", "-C", str(odir), f"-j{min(16, os.cpu_count() or 4)}", *extra, *targets]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"[build] oracle targets {targets}", file=sys.stderr)


if __name__ == "__main__":
    build_library(verbose=True)
    build_oracle(verbose=True)
