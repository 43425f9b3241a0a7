"""The drop-in host's ingest and output (raptor_gb300/host), checked without
a GPU: the C dump reader against the Python reader, and the image/spectrum
writer byte for byte against files written by the reference's own
output_files (tests/golden/ref_output, made by make_golden.py)."""
import os
import subprocess

import numpy as np
import pytest

from raptor_gb300 import harm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "raptor_gb300", "host")
GOLD = os.path.join(ROOT, "tests", "golden", "ref_output")


@pytest.fixture(scope="module")
def host_check(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("hc") / "host_check")
    subprocess.run(["gcc", "-O2", "-std=c11", "-fopenmp", "-I" + os.path.join(ROOT, "include"), "-I" + HOST,
                    os.path.join(ROOT, "tests", "host_check.c"), os.path.join(HOST, "harm_io.c"),
                    os.path.join(HOST, "model_io.c"), "-lm", "-o", exe], check=True)
    return exe


def _parse(exe, path, out):
    r = subprocess.run([exe, "parse", str(path), str(out)], capture_output=True, text=True)
    return r


def test_c_reader_matches_python_reader(host_check, tmp_path, torus64):
    p = tmp_path / "d.dump"
    harm.write_dump(p, torus64)
    r = _parse(host_check, p, tmp_path / "prims.bin")
    assert r.returncode == 0, r.stderr
    raw = open(tmp_path / "prims.bin", "rb").read()
    n1, n2 = np.frombuffer(raw[:8], dtype=np.int32)
    prims = np.frombuffer(raw[8:], dtype=np.float64).reshape(8, n1, n2)
    assert (n1, n2) == (64, 64)
    assert np.array_equal(prims, torus64.prims)


def test_c_reader_sequential_path(host_check, tmp_path, torus64):
    """Records not one per line (fscanf does not care) take the token path."""
    p = tmp_path / "d.dump"
    harm.write_dump(p, torus64)
    txt = open(p).read().split("\n")
    joined = txt[0] + "\n" + " ".join(txt[1:])
    (tmp_path / "j.dump").write_text(joined)
    r = _parse(host_check, tmp_path / "j.dump", tmp_path / "prims.bin")
    assert r.returncode == 0, r.stderr
    prims = np.frombuffer(open(tmp_path / "prims.bin", "rb").read()[8:]).reshape(8, 64, 64)
    assert np.array_equal(prims, torus64.prims)


def test_c_reader_rejects_bad_dumps(host_check, tmp_path, torus64):
    p = tmp_path / "d.dump"
    harm.write_dump(p, torus64)
    lines = open(p).read().splitlines()
    (tmp_path / "t.dump").write_text("\n".join(lines[:500]) + "\n")
    r = _parse(host_check, tmp_path / "t.dump", tmp_path / "o.bin")
    assert r.returncode != 0 and "short" in r.stderr
    bad = lines[:]
    f = bad[7].split()
    f[5] = "nan"
    bad[7] = " ".join(f)
    (tmp_path / "n.dump").write_text("\n".join(bad) + "\n")
    r = _parse(host_check, tmp_path / "n.dump", tmp_path / "o.bin")
    assert r.returncode != 0 and "non-finite" in r.stderr
    hdr = lines[0].split()
    hdr[1] = "1"
    (tmp_path / "h.dump").write_text(" ".join(hdr) + "\n" + "\n".join(lines[1:]) + "\n")
    r = _parse(host_check, tmp_path / "h.dump", tmp_path / "o.bin")
    assert r.returncode != 0


def test_output_files_byte_identical_to_reference(host_check, tmp_path):
    from tests.parity import load_golden
    z = load_golden("small_g64.npz")
    img = np.ascontiguousarray(z["g64_i60_rk4_img"], dtype=np.float64)
    spec = z["g64_i60_rk4_spec"][0]
    img.tofile(tmp_path / "field.bin")
    model = harm.ModelIn.read(os.path.join(GOLD, "model.in"))
    model.write(tmp_path / "model.in")
    r = subprocess.run([host_check, "write", str(tmp_path / "field.bin"), repr(float(spec)), "model.in",
                        "torus64.dump", "1e19", "60", "3", "3", "1"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for fn in os.listdir(GOLD):
        if fn.startswith("img_data"):
            assert open(tmp_path / "output" / fn, "rb").read() == open(os.path.join(GOLD, fn), "rb").read(), fn
        elif fn.startswith("spectrum"):
            # 16 significant digits of JANSKY_FACTOR * spectrum: the reference
            # is built with -Ofast, whose reassociation can move the last digit
            got = np.loadtxt(tmp_path / "output" / fn)
            want = np.loadtxt(os.path.join(GOLD, fn))
            np.testing.assert_allclose(got, want, rtol=1e-14)
    assert sorted(os.listdir(tmp_path / "output")) == sorted(f for f in os.listdir(GOLD) if f != "model.in")


def test_host_program_usage():
    from raptor_gb300 import build
    exe = build.build_host()
    if not exe:
        pytest.skip("host sources missing")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stderr
