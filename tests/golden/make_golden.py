"""Generate the golden fixtures in tests/golden/ (run in the build container).

1. dscaex.json -- the reference's known-answer system EXAMPLE/DSCAEXMAT.dat
   (6x6 A) and EXAMPLE/DSCAEXRHS.dat (b), read in the PDLAREAD format (first
   line "M N", then values in column-major order), together with its exact
   solution computed in rational arithmetic.  EXAMPLE/pdscaex.f:181-191 accepts
   a solve when ||A x - b|| / (||A|| ||x|| eps N) < 10.
2. pdmatgen.json -- leading values of the LU tester's generator for the seeds
   the tester uses (IASEED=100, IBSEED=200, TESTING/traditional/LIN/
   pdludriver.f:130-131), computed with a transcription of the Fortran integer
   routines LMUL / LADD / XJUMPM / PDRAND (TESTING/traditional/LIN/
   pmatgeninc.f) that keeps the 16-bit/15-bit halves exactly as the Fortran
   does.  This is independent of the C oracle's 64-bit jump-ahead arithmetic,
   so the test that compares the two pins the oracle's generator.

Usage: python tests/golden/make_golden.py /path/to/reference-tree
"""
from __future__ import annotations

import json
import os
import sys
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py /path/to/reference-tree (the ScaLAPACK source tree)")
REF = sys.argv[1]


def read_pdlaread(path):
    with open(path) as f:
        toks = f.read().split()
    m, n = int(toks[0]), int(toks[1])
    vals = [float(t.replace("D", "E").replace("d", "e")) for t in toks[2:2 + m * n]]
    return m, n, vals


def solve_exact(n, a_colmajor, b):
    A = [[Fraction(a_colmajor[i + j * n]).limit_denominator(10**12) for j in range(n)] for i in range(n)]
    x = [Fraction(v).limit_denominator(10**12) for v in b]
    # Gaussian elimination with exact rationals
    for k in range(n):
        p = next(i for i in range(k, n) if A[i][k] != 0)
        A[k], A[p] = A[p], A[k]
        x[k], x[p] = x[p], x[k]
        for i in range(k + 1, n):
            f = A[i][k] / A[k][k]
            for j in range(k, n):
                A[i][j] -= f * A[k][j]
            x[i] -= f * x[k]
    for k in range(n - 1, -1, -1):
        s = x[k] - sum(A[k][j] * x[j] for j in range(k + 1, n))
        x[k] = s / A[k][k]
    return x


# ---- PDRAND in the Fortran's own two-halves integer arithmetic ----
IPOW15, IPOW16, IPOW30 = 2**15, 2**16, 2**30


def lmul(k, j):
    kt = k[0] * j[0]
    if kt < 0:
        kt = (kt + IPOW30) + IPOW30
    i0 = kt % IPOW16
    lt = k[0] * j[1] + k[1] * j[0]
    if lt < 0:
        lt = (lt + IPOW30) + IPOW30
    kt = kt // IPOW16 + lt
    if kt < 0:
        kt = (kt + IPOW30) + IPOW30
    return [i0, kt % IPOW15]


def ladd(j, k):
    return [(k[0] + j[0]) % IPOW16, ((k[0] + j[0]) // IPOW16 + k[1] + j[1]) % IPOW15]


def pdrand_stream(seed, count):
    mult = [20077, 16838]
    iadd = [12345, 0]
    # XJUMPM(1, MULT, IADD, JSEED, IRAN1, IA1, IC1): IRAN1 = MULT*JSEED + IADD
    iran = ladd(lmul([seed, 0], mult), iadd)
    out = []
    for _ in range(count):
        out.append((iran[0] + 65536.0 * iran[1]) / 2147483648.0)
        iran = ladd(lmul(iran, mult), iadd)
    return out


def main():
    m, n, a = read_pdlaread(os.path.join(REF, "EXAMPLE", "DSCAEXMAT.dat"))
    mb, nbr, b = read_pdlaread(os.path.join(REF, "EXAMPLE", "DSCAEXRHS.dat"))
    assert m == n == mb and nbr == 1
    x = solve_exact(n, a, b)
    with open(os.path.join(HERE, "dscaex.json"), "w") as f:
        json.dump({
            "source": "EXAMPLE/DSCAEXMAT.dat, EXAMPLE/DSCAEXRHS.dat (PDLAREAD format)",
            "n": n, "nrhs": 1, "nb": 2,
            "a_colmajor": a, "b": b,
            "x_exact": [float(v) for v in x],
            "x_exact_fraction": [str(v) for v in x],
            "threshold": 10.0,
        }, f, indent=1)
    gen = {"source": "TESTING/traditional/LIN/pmatgeninc.f PDRAND via LMUL/LADD", "values": {}}
    for seed in (100, 200, 1, 12345):
        gen["values"][str(seed)] = pdrand_stream(seed, 64)
    with open(os.path.join(HERE, "pdmatgen.json"), "w") as f:
        json.dump(gen, f, indent=1)
    print("wrote", os.path.join(HERE, "dscaex.json"), os.path.join(HERE, "pdmatgen.json"))


if __name__ == "__main__":
    main()
