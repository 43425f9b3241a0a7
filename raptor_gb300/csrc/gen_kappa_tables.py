"""Generate kappa_tables.inc: the power-series coefficients of the two Gauss
hypergeometric functions the kappa-distribution absorptivity needs
(kappa.cuh), each coefficient correctly rounded to double.

    python raptor_gb300/csrc/gen_kappa_tables.py

The absorptivity fit (j_nu.c:56-106, kappa = 3.5 as hard-coded there)
evaluates 2F1(a, b; c; z) with a = kappa - 1/3, b = kappa + 1,
c = kappa + 2/3 and z = -kappa Theta_e < 0.  For |z| <= 1 the engine uses
Pfaff's transformation 2F1(a, b; c; z) = (1 - z)^-a 2F1(a, c - b; c; x),
x = z / (z - 1) in [0, 1/2]; for |z| > 1 the reference's own connection
formula, whose second function is 2F1(b, c - a; b - a + 1; w),
w = 1 / (1 - z) in (0, 1/2) (its first, 2F1(a, c - b; a - b + 1; w), is
(1 - w)^-a because c - b = a - b + 1).  With x, w <= 1/2 both power series
sum_n (p)_n (q)_n / ((r)_n n!) x^n are within 1e-18 of their limits after
80 terms.  The coefficients are exact rationals here (Python fractions),
then rounded.  The FP32 samples of the mixed forms take the first 40 terms
rounded to FP32 (kKappaPfaffF, kKappaConnF): after 40 terms the series are
within 1e-9 of their limits, below FP32's rounding."""
import os
import struct
from fractions import Fraction

KAPPA = Fraction(7, 2)
N_TERMS = 80
N_TERMS_F32 = 40


def to_f32(v):
    """v rounded to FP32 (through its double), as a C float literal."""
    f = struct.unpack("f", struct.pack("f", float(v)))[0]
    t = f"{f:.9g}"
    return (t if ("." in t or "e" in t) else t + ".0") + "f"


def coefficients(p, q, r, n_terms=N_TERMS):
    """(p)_n (q)_n / ((r)_n n!), n = 0 .. n_terms - 1, exact."""
    out, c = [], Fraction(1)
    for n in range(n_terms):
        out.append(c)
        c = c * (p + n) * (q + n) / ((r + n) * (n + 1))
    return out


def series():
    a, b, c = KAPPA - Fraction(1, 3), KAPPA + 1, KAPPA + Fraction(2, 3)
    # (name, p, q, r, comment)
    return [
        ("kKappaPfaff", a, c - b, c, "2F1(a, c - b; c; x), x = z / (z - 1) in [0, 1/2]"),
        ("kKappaConn", b, c - a, b - a + 1, "2F1(b, c - a; b - a + 1; w), w = 1 / (1 - z) in (0, 1/2)"),
    ]


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    lines = ["// Generated by gen_kappa_tables.py - do not edit.", ""]
    for name, p, q, r, what in series():
        lines.append(f"// {what}: coefficient n of the power series, p = {p}, q = {q}, r = {r}")
        lines.append(f"__device__ const double {name}[{N_TERMS}] = {{")
        lines += [f"    {float(v)!r}," for v in coefficients(p, q, r)]
        lines.append("};")
        lines.append("")
    for name, p, q, r, what in series():
        lines.append(f"// the same, first {N_TERMS_F32} coefficients rounded to FP32")
        lines.append(f"__device__ const float {name}F[{N_TERMS_F32}] = {{")
        lines += [f"    {to_f32(v)}," for v in coefficients(p, q, r, N_TERMS_F32)]
        lines.append("};")
        lines.append("")
    with open(os.path.join(here, "kappa_tables.inc"), "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main()
