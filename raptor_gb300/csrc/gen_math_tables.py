"""Generate the tables of the table-driven exp and sincospi:
math_tables.inc (fp64_math.cuh, each entry correctly rounded to double) and
df_tables.inc (df64.cuh, each entry as an unevaluated pair hi + lo of FP32
numbers, hi the value rounded to FP32 and lo the remainder rounded to FP32).

    python raptor_gb300/csrc/gen_math_tables.py

Values are computed with Python's decimal module at 50 significant digits
(Taylor series), then rounded."""
import os
import struct
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


def sincospi_entry(n, half):
    """sin and cos of pi n / half, exact at the multiples of pi/2, where the
    series of the truncated pi leaves residues of order 1e-46 instead of 0."""
    if (2 * n) % half == 0:
        return [(Decimal(0), Decimal(1)), (Decimal(1), Decimal(0)),
                (Decimal(0), Decimal(-1)), (Decimal(-1), Decimal(0))][(2 * n // half) % 4]
    return dsincos(PI * n / half)


def f32(x):
    """Round a Decimal to the nearest FP32 value (through an exact double
    near it; a double-rounding tie changes hi by one ulp and lo absorbs it)."""
    return struct.unpack("f", struct.pack("f", float(x)))[0]


def split(x):
    hi = f32(x)
    lo = f32(x - Decimal(hi))
    return hi, lo


def ffmt(v):
    return f"{v!r}f" if v != 0 else "0.0f"


def write_df_tables(here):
    lines = ["// Generated by gen_math_tables.py - do not edit.", "",
             "// 2^(j/64) as (hi, lo) FP32 pairs, j = 0..63", "__device__ const float2 kExp2TableDF[64] = {"]
    for j in range(64):
        hi, lo = split(dexp(LN2 * j / 64))
        lines.append(f"    {{{ffmt(hi)}, {ffmt(lo)}}},")
    lines.append("};")
    lines += ["", "// (sin hi, sin lo, cos hi, cos lo) of pi n/128, n = 0..255",
              "__device__ const float4 kSinCosPiTableDF[256] = {"]
    for n in range(256):
        s, c = sincospi_entry(n, 128)
        sh, sl = split(s)
        ch, cl = split(c)
        lines.append(f"    {{{ffmt(sh)}, {ffmt(sl)}, {ffmt(ch)}, {ffmt(cl)}}},")
    lines.append("};")
    # constants: pi, ln2/64 split for Cody-Waite reduction, 1/6
    pih, pil = split(PI)
    l2 = LN2 / 64
    # L1 with 12 significant bits so that n * L1 is exact for |n| < 2^12
    e = 0
    while Decimal(2) ** (e + 1) <= l2:
        e += 1
    while Decimal(2) ** e > l2:
        e -= 1
    q = Decimal(2) ** (e - 11)
    L1 = (l2 / q).to_integral_value(rounding="ROUND_FLOOR") * q
    L2 = f32(l2 - L1)
    L3 = f32(l2 - L1 - Decimal(L2))
    sxh, sxl = split(Decimal(1) / 6)
    lines += ["", f"constexpr float kPiDFhi = {ffmt(pih)}, kPiDFlo = {ffmt(pil)};",
              f"constexpr float kLn2by64_1 = {ffmt(f32(L1))};  // 12 significant bits",
              f"constexpr float kLn2by64_2 = {ffmt(L2)}, kLn2by64_3 = {ffmt(L3)};",
              f"constexpr float kSixthDFhi = {ffmt(sxh)}, kSixthDFlo = {ffmt(sxl)};"]
    open(os.path.join(here, "df_tables.inc"), "w").write("\n".join(lines) + "\n")


def main():
    write_df_tables(os.path.dirname(os.path.abspath(__file__)))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "math_tables.inc")
    lines = ["// Generated by gen_math_tables.py - do not edit.", "",
             "// 2^(j/128), j = 0..127", "__device__ const double kExp2Table[128] = {"]
    for j in range(128):
        lines.append(f"    {float(dexp(LN2 * j / 128))!r},")
    lines.append("};")
    lines += ["", "// (sin(pi n/512), cos(pi n/512)), n = 0..1023 (period 2 in the argument)",
              "__device__ const double2 kSinCosPiTable[1024] = {"]
    for n in range(1024):
        s, c = sincospi_entry(n, 512)
        lines.append(f"    {{{float(s)!r}, {float(c)!r}}},")
    lines.append("};")
    open(out, "w").write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
