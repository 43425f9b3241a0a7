"""The integration patch of INTEGRATION.md section 1 compiles: the
reference's own core.c (core.c:74-152, declared at functions.h:70) with
calculate_image replaced by the engine call, built with the rest of the
reference program and linked against libraptor_gpu.so (CPU: link only,
nothing runs).  tests/test_gpu_integration_patch.py runs the result."""
import os

import pytest

from tests import integration_patch as ip


def test_patch_replaces_only_calculate_image():
    src = ip.sources_dir()
    if src is None:
        pytest.skip("the reference's sources are not staged on this machine")
    core = open(os.path.join(src, "core.c")).read()
    out = ip.patched_core(core, ip.patch_block())
    # the patched file keeps every other function of core.c
    for fn in ("void read_model(", "void output_files(", "void write_image("):
        if fn in core:
            assert out.count(fn) == core.count(fn), fn
    assert out.count("void calculate_image(") == 1 and "raptor_gpu_render(" in out
    assert "integrate_geodesic(" not in out[out.index("void calculate_image("):]
    # everything before calculate_image is untouched, everything after it too
    assert out.startswith(core[:core.index("void calculate_image(")])
    assert out.endswith(core[core.index("void output_files("):])


def test_patched_reference_program_links(tmp_path):
    from raptor_gb300 import build, engine
    if ip.sources_dir() is None:
        pytest.skip("the reference's sources are not staged on this machine")
    if not os.path.exists(engine.LIB_PATH):
        build.build_library()
    exe = ip.build(str(tmp_path))
    assert os.access(exe, os.X_OK)
