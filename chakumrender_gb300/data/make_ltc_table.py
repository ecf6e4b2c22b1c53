"""Converts the reference's GGX LTC fit tables (headers/ltc.inc) into ltc_ggx.bin.

The table has to be identical to the reference's for parity: it is fitted data (the
linearly transformed cosine fits of Heitz et al. 2016 as shipped by the reference),
not code.  Run from the repo root where the reference is available:

    python chakumrender_gb300/data/make_ltc_table.py /path/to/reference/headers/ltc.inc

Output layout (little-endian):
    8 bytes   magic b"CKRLTC1\\0"
    int32     size (64), int32 reserved (0)
    float64   tabM[size*size][9]      as written in ltc.inc (row order m0..m8)
    float64   tabMinv[size*size][9]
    float32   tabAmplitude[size*size]
The decimal literals are parsed with correct rounding, as a C compiler parses them
(doubles for the matrices, floats for the amplitudes).
"""
from __future__ import annotations

import re
import struct
import sys
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "ltc_ggx.bin"
NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?"


def block(text: str, name: str) -> str:
    m = re.search(name + r"\s*\[[^\]]*\]\s*=\s*\{(.*?)\};", text, re.S)
    if not m:
        raise SystemExit(f"table {name} not found")
    return m.group(1)


def main(src: str) -> None:
    text = Path(src).read_text()
    size = int(re.search(r"static const int size\s*=\s*(\d+)", text).group(1))
    n = size * size
    tm = np.array([float(x) for x in re.findall(NUM, block(text, "tabM"))], dtype=np.float64)
    ti = np.array([float(x) for x in re.findall(NUM, block(text, "tabMinv"))], dtype=np.float64)
    amp_txt = re.findall(NUM + r"f?", block(text, "tabAmplitude"))
    ta = np.array([np.float32(s.rstrip("f")) for s in amp_txt], dtype=np.float32)
    assert tm.size == 9 * n and ti.size == 9 * n and ta.size == n, (tm.size, ti.size, ta.size)
    with open(OUT, "wb") as f:
        f.write(b"CKRLTC1\0")
        f.write(struct.pack("<ii", size, 0))
        f.write(tm.astype("<f8").tobytes())
        f.write(ti.astype("<f8").tobytes())
        f.write(ta.astype("<f4").tobytes())
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {n} entries)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_ltc_table.py <reference checkout>/headers/ltc.inc")
    main(sys.argv[1])
