"""The same-named C++ API (include/ckr_dropin.hpp) and the main() programs of
INTEGRATION.md section 1 compile and link against libckr.so.  No GPU: the programs
are built, not run (tests/test_dropin_gpu.py runs them)."""
from __future__ import annotations

import dropin_build as D


def test_integration_programs_and_queries_compile(tmp_path):
    exes = D.build_all(tmp_path)
    for name, exe in exes.items():
        assert exe.exists(), name


def test_integration_section_1_has_both_programs():
    progs = D.integration_programs()
    assert "ckr_dropin.hpp" in progs["dropin_main"] and "shade(rays.data()" in progs["dropin_main"]
    for call in ("initSceneParser", "prepareScreenCamera", "prepareObjects", "prepareLightSources", "loadAccels",
                 "loadLightSampler"):
        assert call + "(" in progs["dropin_main"], call
    assert "ckr_render_host" in progs["cabi_main"]
