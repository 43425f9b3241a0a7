"""The reference RAPTOR program with the integration patch of INTEGRATION.md
section 1 applied to its core.c (tests/integration_patch.py), run on the GPU
with the reference's command line: its own read_model, init_model (the HARM
dump reader), set_constants and output_files around the engine.  Its output
files are compared with the files the unpatched reference wrote for the same
image (tests/golden/ref_output: 32x32, i = 60, 230 GHz, 64x64 torus)."""
import os
import subprocess

import numpy as np
import pytest

from raptor_gb300 import harm
from tests import integration_patch as ip

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_patched_reference_reproduces_its_files(tmp_path, torus64):
    if ip.sources_dir() is None:
        pytest.skip("the reference's sources are not staged on this machine")
    gold = os.path.join(ROOT, "tests", "golden", "ref_output")
    exe = ip.build(str(tmp_path / "build"), n1=64, n2=64, rk="RK4")
    run = tmp_path / "run"
    run.mkdir()
    harm.write_dump(run / "torus64.dump", torus64)
    harm.ModelIn.read(os.path.join(gold, "model.in")).write(run / "model.in")
    r = subprocess.run([exe, "model.in", "torus64.dump", "1e19", "60", "3", "3", "1"], cwd=run,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
    for fn in os.listdir(gold):
        if fn == "model.in":
            continue
        got = open(run / "output" / fn).read().splitlines()
        want = open(os.path.join(gold, fn)).read().splitlines()
        assert len(got) == len(want), fn
        if fn.startswith("img_data"):
            # the header names the dump file as given on the command line
            assert got[0].split()[:4] == want[0].split()[:4], "header"
            g = np.array([float(x) for x in got[1:]])
            w = np.array([float(x) for x in want[1:]])
            # six significant digits per pixel (utilities.c:61): identical
            # except where last-bit differences straddle a rounding boundary
            differ = int(np.sum(np.array(got[1:]) != np.array(want[1:])))
            assert differ <= 2, f"{differ} of {len(w)} pixel lines differ"
            np.testing.assert_allclose(g, w, rtol=1e-5, atol=0)
        else:
            np.testing.assert_allclose(np.loadtxt(run / "output" / fn), np.loadtxt(os.path.join(gold, fn)),
                                       rtol=1e-6)
