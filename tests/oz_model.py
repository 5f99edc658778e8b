"""numpy model of the sliced FP64 product's scales (scalapack_gb300/csrc/
ozgemm_f64.cu): the power-of-two balancing along k, the row and column scale
exponents, and the error-budget test that sends a pass to the FP64 route.
Shared by the CPU model tests and the GPU product tests."""
from __future__ import annotations

import numpy as np

BUDGET = 8  # bits (OZ_BUDGET)


def _ex(x):
    """frexp exponents of |x| (|x| < 2^ex), 0 where x is zero or not finite."""
    a = np.abs(np.asarray(x, dtype=np.float64))
    ok = np.isfinite(a) & (a > 0)
    e = np.frexp(np.where(ok, a, 1.0))[1].astype(np.int64)
    return np.where(ok, e, 0), ok


def scales(A, B, balance=True, side="A"):
    """One pass (k <= 256) of C += A B: returns (e, f, tripped, info).

    side "A" (the default) balances by the columns of A (d_k = c_k) and tests
    the error budget per row; side "B" balances by the rows of B (d_k = -h_k)
    and tests it per column. e[i], f[j]: the scale exponents (None for a row /
    column without an active nonzero); tripped: the pass takes the FP64 route;
    info: c, h, G, F, gap. With balance=False the scales are the plain row /
    column maxima (the product before the balancing), for comparison."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    EA, okA = _ex(A)
    EB, okB = _ex(B)
    hasB = okB.any(axis=1)
    hasA = okA.any(axis=0)
    lo = -10 ** 6
    h = np.where(hasB, np.max(np.where(okB, EB, lo), axis=1), 0)
    c = np.where(hasA, np.max(np.where(okA, EA, lo), axis=0), 0)
    active = hasA & hasB
    d = (c if side == "A" else -h) if balance else np.zeros_like(c)
    big = -10 ** 9
    e = np.where(okA & active[None, :], EA - d[None, :], big).max(axis=1)
    f = np.where(okB & active[:, None], EB + d[:, None], big).max(axis=0)
    G = np.where(active, c + h, big).max() if active.any() else big
    if side == "A":
        F = np.where(okA & active[None, :], EA + h[None, :], big).max(axis=1)
        gap = np.where(e > big, e + G - F, 0)
    else:
        F = np.where(okB & active[:, None], c[:, None] + EB, big).max(axis=0)
        gap = np.where(f > big, f + G - F, 0)
    e_l = [int(v) if v > big else None for v in e]
    f_l = [int(v) if v > big else None for v in f]
    in_range = all(v is None or -1022 <= v - 26 <= 1023 for v in e_l + f_l)
    tripped = bool(np.any(gap > BUDGET)) or not in_range
    return e_l, f_l, tripped, dict(c=c, h=h, G=G, F=F, gap=gap)


def bound_gap_bits(A, B, balance=True, side="A"):
    """Largest excess, in bits, of the error scale 2^(e_i + f_j) over the
    largest term max_k |A(i,k) B(k,j)| of each entry (entries whose terms are
    all zero are skipped): the componentwise price of the slicing."""
    e, f, _, _ = scales(A, B, balance=balance, side=side)
    T = np.max(np.abs(A)[:, :, None] * np.abs(B)[None, :, :], axis=1)
    worst = -np.inf
    for i, ei in enumerate(e):
        for j, fj in enumerate(f):
            if ei is None or fj is None or T[i, j] == 0:
                continue
            worst = max(worst, ei + fj - np.log2(T[i, j]))
    return worst


def graded_lu_operands(rng, m, k, n, spread):
    """L21 / U12 of a row-graded LU step: rows of A scaled by 2^s_i, the
    pivot rows of the block the k largest; L(i,k) = l 2^(s_i - s_pk) (<= 1),
    U(k,j) = u 2^(s_pk)."""
    s_piv = np.sort(rng.integers(-spread, spread + 1, size=k))[::-1]
    s_row = rng.integers(-spread, int(s_piv.min()) + 1, size=m)
    L = rng.uniform(-1, 1, (m, k)) * np.exp2(s_row[:, None] - s_piv[None, :])
    L = np.clip(L, -1.0, 1.0)
    U = rng.uniform(-1, 1, (k, n)) * np.exp2(s_piv[:, None])
    return L, U


def graded_inverse_operands(rng, k, n, spread):
    """The U12 solve's product on a row-graded block: A = inv(L_bb) - I of a
    unit-lower 64-row block whose pivots decrease in size, B = the block's
    rows of A12 (scaled like their pivots). Side B's case."""
    s = np.sort(rng.integers(-spread, spread + 1, size=k))[::-1]
    L = np.tril(rng.uniform(-1, 1, (k, k)) * np.exp2(s[:, None] - s[None, :]), -1) + np.eye(k)
    Ninv = np.linalg.inv(L) - np.eye(k)
    B = rng.uniform(-1, 1, (k, n)) * np.exp2(s[:, None])
    return Ninv, B


def spike_operands(rng, m, k, n, big=40, tiny=-50):
    """Row 0 of B holds one entry 2^big above the rest, and row 0 of A is
    2^tiny small in column 0: the product's row 0 needs the k = 0 term at
    full precision although row 0's scale is set by the other k. No
    balancing helps; the row budget test sends the pass to the FP64 route."""
    A = rng.uniform(-1, 1, (m, k))
    B = rng.uniform(-1, 1, (k, n))
    B[0, n // 2] = 2.0 ** big
    A[0, 0] = 2.0 ** tiny
    return A, B
