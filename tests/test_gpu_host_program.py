"""The drop-in host program end to end on the GPU: the reference's command
line, model.in and HARM dump in, the reference's output files out, compared
with files the reference itself wrote for the same image
(tests/golden/ref_output: 32x32, i = 60, 230 GHz, 64x64 torus;
tests/golden/ref_output_logcam: the same through a LOG_IMPACT_CAM build,
32x24)."""
import os
import subprocess

import numpy as np
import pytest

from raptor_gb300 import harm

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

@pytest.mark.parametrize("gold_name,camera", [("ref_output", "linear"), ("ref_output_logcam", "log")])
def test_host_program_reproduces_reference_files(tmp_path, torus64, gold_name, camera):
    from raptor_gb300 import build
    GOLD = os.path.join(ROOT, "tests", "golden", gold_name)
    exe = build.build_host()
    assert exe
    harm.write_dump(tmp_path / "torus64.dump", torus64)
    harm.ModelIn.read(os.path.join(GOLD, "model.in")).write(tmp_path / "model.in")
    env = dict(os.environ, RAPTOR_INT_METHOD="RK4", RAPTOR_PRECISION="fp64", RAPTOR_CAMERA=camera)
    r = subprocess.run([exe, "model.in", "torus64.dump", "1e19", "60", "3", "3", "1"], cwd=tmp_path, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    for fn in os.listdir(GOLD):
        if fn == "model.in":
            continue
        got = open(tmp_path / "output" / fn).read().splitlines()
        want = open(os.path.join(GOLD, fn)).read().splitlines()
        assert len(got) == len(want), fn
        if fn.startswith("img_data"):
            assert got[0] == want[0], "header"
            g = np.array([float(x) for x in got[1:]])
            w = np.array([float(x) for x in want[1:]])
            # six significant digits per pixel: identical except where the
            # engine's last-bit differences straddle a rounding boundary
            differ = np.sum(np.array(got[1:]) != np.array(want[1:]))
            assert differ <= 2, f"{differ} of {len(w)} pixel lines differ"
            np.testing.assert_allclose(g, w, rtol=1e-5, atol=0)
        else:
            np.testing.assert_allclose(np.loadtxt(tmp_path / "output" / fn), np.loadtxt(os.path.join(GOLD, fn)),
                                       rtol=1e-6)
