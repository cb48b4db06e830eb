"""Generate voigt_table.h: real-axis values of the Faddeeva function w(x).

For x_j = j * 0.1 (j = 0 .. 120) the table holds, to full double precision,
  E_j = exp(-x_j^2),
  D_j = (2/sqrt(pi)) F(x_j),            F = Dawson's integral,
  G_j = (2/sqrt(pi)) (1 - 2 x_j F(x_j)) = (2/sqrt(pi)) F'(x_j),
so that w(x_j) = E_j + i D_j and w'(x_j) = -2 x_j E_j + i G_j.  The device
code expands w(z) in a Taylor series about the nearest x_j using the ODE
w'(z) = -2 z w(z) + 2i/sqrt(pi).  Values are computed with mpmath at 60 digits
and written as exact hexadecimal float literals.  Run once at development time
(needs mpmath); the generated header is committed.

The header also holds the table of the FP32 small-damping form: to first
order in the damping a (error O(a^2) relative, below 6e-7 for a <= 2e-3),
    H(a, x) = exp(-x^2) (1 + a^2 (1 - 2 x^2)) + a K(x),
    K(x) = -(2/sqrt(pi)) (1 - 2 x F(x)) = -G(x),
with K on [0, 16) as one cubic per interval of 0.1: the cubic Hermite
interpolant of K and K' = -(2/sqrt(pi)) (-2 F - 2 x F') at the interval ends,
as float coefficients {c0, c1, c2, c3} of p(t) = c0 + c1 t + c2 t^2 + c3 t^3,
t = (x - x_j) / 0.1 (interpolation error below 2.3e-7 of H, checked against
scipy's wofz).
"""
import os
import mpmath as mp

mp.mp.dps = 60
H = mp.mpf(1) / 10
N = 121


def dawson(x):
    return mp.sqrt(mp.pi) / 2 * mp.exp(-x * x) * mp.erfi(x)


KN = 160   # intervals of the small-damping table, [0, 16)


def ktab_rows():
    c = 2 / mp.sqrt(mp.pi)

    def k_and_dk(x):
        F = dawson(x)
        dF = 1 - 2 * x * F
        return -c * (1 - 2 * x * F), -c * (-2 * F - 2 * x * dF)

    rows = []
    for j in range(KN):
        y0, d0 = k_and_dk(j * H)
        y1, d1 = k_and_dk((j + 1) * H)
        d0 *= H
        d1 *= H
        coef = (y0, d0, -3 * y0 - 2 * d0 + 3 * y1 - d1, 2 * y0 + d0 - 2 * y1 + d1)
        rows.append(tuple(float(mp.mpf(v)).hex() for v in coef))
    return rows


def main():
    rows = []
    for j in range(N):
        x = j * H
        F = dawson(x)
        c = 2 / mp.sqrt(mp.pi)
        vals = (mp.exp(-x * x), c * F, c * (1 - 2 * x * F))
        rows.append(tuple(float(v).hex() for v in vals))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "voigt_table.h")
    with open(out, "w") as f:
        f.write("/* Generated by gen_voigt_table.py -- do not edit.\n"
                " * Real-axis Faddeeva data at x_j = j/10: {exp(-x^2), 2/sqrt(pi) F(x),\n"
                " * 2/sqrt(pi) (1 - 2 x F(x))}, F = Dawson's integral. */\n")
        f.write("#pragma once\n#define FSG_VTAB_N %d\n#define FSG_VTAB_H 0.1\n" % N)
        f.write("#define FSG_VTAB_INVH 10.0\n")
        f.write("/* rows padded to 4 doubles (32 bytes) for two aligned 16-byte loads */\n")
        f.write("#define FSG_VTAB_INIT { \\\n")
        for r in rows:
            f.write("    {%s, %s, %s, 0.0}, \\\n" % r)
        f.write("}\n")
        f.write("/* Small-damping form: cubic coefficients {c0, c1, c2, c3} of\n"
                " * K(x) = -(2/sqrt(pi)) (1 - 2 x F(x)) on [j/10, (j+1)/10), t = 10 x - j. */\n")
        f.write("#define FSG_KTAB_N %d\n" % KN)
        f.write("#define FSG_KTAB_INIT { \\\n")
        for r in ktab_rows():
            f.write("    {%sf, %sf, %sf, %sf}, \\\n" % r)
        f.write("}\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
