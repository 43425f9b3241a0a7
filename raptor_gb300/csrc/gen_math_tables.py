"""Generate math_tables.inc: the tables of the table-driven FP64 exp and
sincospi in fp64_math.cuh, each entry correctly rounded to double.

    python raptor_gb300/csrc/gen_math_tables.py

Values are computed with Python's decimal module at 50 significant digits
(Taylor series), then rounded once to the nearest double."""
import os
from decimal import Decimal, getcontext

getcontext().prec = 50
PI = Decimal("3.14159265358979323846264338327950288419716939937510")
LN2 = Decimal("0.69314718055994530941723212145817656807550013436026")


def dexp(x):
    s, t, k = Decimal(1), Decimal(1), 1
    while True:
        t = t * x / k
        if abs(t) < Decimal("1e-45"):
            return s + t
        s += t
        k += 1


def dsincos(x):
    s, c = Decimal(0), Decimal(0)
    t, k = Decimal(1), 0
    while True:
        if k % 4 == 0:
            c += t
        elif k % 4 == 1:
            s += t
        elif k % 4 == 2:
            c -= t
        else:
            s -= t
        k += 1
        t = t * x / k
        if abs(t) < Decimal("1e-45") and k > 4:
            return s, c


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "math_tables.inc")
    lines = ["// Generated by gen_math_tables.py - do not edit.", "",
             "// 2^(j/64), j = 0..63", "__device__ const double kExp2Table[64] = {"]
    for j in range(64):
        lines.append(f"    {float(dexp(LN2 * j / 64))!r},")
    lines.append("};")
    lines += ["", "// (sin(pi n/128), cos(pi n/128)), n = 0..255 (period 2 in the argument)",
              "__device__ const double2 kSinCosPiTable[256] = {"]
    for n in range(256):
        s, c = dsincos(PI * n / 128)
        lines.append(f"    {{{float(s)!r}, {float(c)!r}}},")
    lines.append("};")
    open(out, "w").write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
