"""The engine's table-driven FP64 exp and sincospi (csrc/fp64_math.cuh)
against CUDA's exp and sincospi, on the GPU: <= 2 ulp, and sin/cos within
2.3e-16 absolute near their zeros (where ulp counts are meaningless).  The
double-float versions (csrc/df64.cuh) against the same FP64 functions:
exp, sin and cos within 2e-14 (a few units of the 48-bit significand), the
division (one correction step, ~2^-45) within 5e-14.  The FP64 reciprocal
(csrc/fp64_math.cuh fast_rcp: the hardware approximation and two
Newton-Raphson steps) within 1 ulp of the IEEE quotient.  The FP32
samples' division and square root (csrc/fp32_math.cuh: PTX div.full.f32 and
sqrt.approx.f32) within 2 ulp and 1 ulp of IEEE division and sqrtf, from
subnormal to near-overflow magnitudes, with IEEE's zeros, infinities and
NaNs.  The integer-pipe double -> float conversion of the mixed adjoint's
tangents (csrc/fp32_math.cuh f32_of) equal to the IEEE conversion from
2^-126 up but at exact ties (1 ulp there), signed zeros below, infinity for
NaN."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fast_math_against_cuda(tmp_path):
    from raptor_gb300 import build
    exe = str(tmp_path / "gpu_math_check")
    subprocess.run([build.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I" + os.path.join(ROOT, "raptor_gb300", "csrc"), os.path.join(ROOT, "tests", "gpu_math_check.cu"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    vals = dict(zip(out[0::2], out[1::2]))
    assert vals["err"] == "no"
    assert float(vals["exp_ulp"]) <= 2
    assert float(vals["sin_abs"]) <= 2.3e-16 and float(vals["cos_abs"]) <= 2.3e-16
    assert float(vals["df_exp_rel"]) <= 2e-14
    assert float(vals["df_sin_abs"]) <= 2e-14 and float(vals["df_cos_abs"]) <= 2e-14
    assert float(vals["df_div_rel"]) <= 5e-14
    assert float(vals["rcp_ulp"]) <= 1
    assert float(vals["fdiv_ulp"]) <= 2 and float(vals["fdiv_sub_ulp"]) <= 2
    assert float(vals["fsqrt_ulp"]) <= 1
    assert vals["f32_special_bad"] == "0"
    assert float(vals["f2f_ulp"]) <= 1 and vals["f2f_bad"] == "0"
