"""The FP64 tables of the table-driven exp and sincospi (csrc/math_tables.inc,
written by csrc/gen_math_tables.py) hold correctly rounded 2^(j/128) and
sin/cos(pi n/512): every entry is re-derived here at 40 significant digits
and must equal the committed double exactly.  The GPU test of the routines
themselves (test_gpu_math.py) checks their accuracy against CUDA's exp and
sincospi."""
import os
import re
from decimal import Decimal, getcontext

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "raptor_gb300", "csrc", "math_tables.inc")


def _array(src, name):
    m = re.search(name + r"\[(\d+)\] = \{(.*?)\};", src, re.S)
    assert m, name
    return int(m.group(1)), m.group(2)


def _exp(x):
    s, t, k = Decimal(1), Decimal(1), 1
    while abs(t) > Decimal("1e-45"):
        t = t * x / k
        s += t
        k += 1
    return s


def _sincos(x):
    s, c, t, k = Decimal(0), Decimal(1), Decimal(1), 1
    while abs(t) > Decimal("1e-45"):
        t = t * x / k
        if k % 4 == 1:
            s += t
        elif k % 4 == 2:
            c -= t
        elif k % 4 == 3:
            s -= t
        else:
            c += t
        k += 1
    return s, c


@pytest.fixture(scope="module")
def src():
    getcontext().prec = 40
    return open(INC).read()


def test_exp_table_correctly_rounded(src):
    n, body = _array(src, "kExp2Table")
    vals = [float(v) for v in body.replace(",", " ").split()]
    assert n == 128 and len(vals) == 128
    ln2 = Decimal("0.6931471805599453094172321214581765680755")
    for j, v in enumerate(vals):
        assert v == float(_exp(ln2 * j / 128)), j


def test_sincospi_table_correctly_rounded(src):
    n, body = _array(src, "kSinCosPiTable")
    pairs = re.findall(r"\{([-0-9.e]+), ([-0-9.e]+)\}", body)
    assert n == 1024 and len(pairs) == 1024
    pi = Decimal("3.141592653589793238462643383279502884197")
    quarter = [(Decimal(0), Decimal(1)), (Decimal(1), Decimal(0)), (Decimal(0), Decimal(-1)), (Decimal(-1), Decimal(0))]
    for k in range(1024):
        # exact at the multiples of pi/2 (the series of a truncated pi leaves ~1e-40 there)
        s, c = quarter[k // 256] if k % 256 == 0 else _sincos(pi * k / 512)
        assert float(pairs[k][0]) == float(s) and float(pairs[k][1]) == float(c), k
