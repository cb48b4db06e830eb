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
"""
import os
import mpmath as mp

mp.mp.dps = 60
H = mp.mpf(1) / 10
N = 121


def dawson(x):
    return mp.sqrt(mp.pi) / 2 * mp.exp(-x * x) * mp.erfi(x)


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
    print("wrote", out)


if __name__ == "__main__":
    main()
