"""The C-ABI library loads and exports every entry point include/raptor_gpu.h
declares (no GPU needed; nothing is computed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "raptor_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(raptor_gpu_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from raptor_gb300 import build, engine
    if not os.path.exists(engine.LIB_PATH):
        build.build_library()
    return ctypes.CDLL(engine.LIB_PATH)


def test_header_declares_the_abi():
    names = declared_functions()
    from raptor_gb300 import engine
    assert set(engine.EXPORTED) <= set(names), names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_struct_layouts_match_header(lib):
    """ctypes mirrors of the ABI structs have the sizes the C compiler gives,
    and every field of the options struct its offset."""
    import subprocess
    import tempfile
    from raptor_gb300 import engine
    opt_fields = [f for f, _ in engine.Options._fields_]
    offs = "".join(f' printf("%zu\\n", offsetof(raptor_gpu_options, {f}));' for f in opt_fields)
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "raptor_gpu.h"
int main(void){printf("%zu %zu %zu %zu %zu\n", sizeof(raptor_gpu_options), sizeof(raptor_grid_geom),
 sizeof(raptor_image_desc), sizeof(raptor_gpu_stats), sizeof(raptor_grad));''' + offs + r'''return 0;}
'''
    d = tempfile.mkdtemp()
    c = os.path.join(d, "s.c")
    open(c, "w").write(src)
    exe = os.path.join(d, "s")
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe], check=True)
    vals = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    sizes, offsets = vals[:5], vals[5:]
    assert sizes == [ctypes.sizeof(engine.Options), ctypes.sizeof(engine.GridGeomC),
                     ctypes.sizeof(engine.ImageDesc), ctypes.sizeof(engine.Stats), ctypes.sizeof(engine.GradC)]
    assert offsets == [getattr(engine.Options, f).offset for f in opt_fields]


def test_init_without_device_fails_cleanly(lib):
    """With no GPU, init reports NODEVICE instead of crashing or exiting."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from raptor_gb300 import engine
    with pytest.raises(engine.EngineError) as e:
        engine.Engine()
    assert e.value.code == -5
