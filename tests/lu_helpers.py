"""Shared helpers for the GPU parity tests: inputs from the tester's generator,
the IPIV comparison with near-tie logging and forced-pivot replay, and the
tester's scaled residuals (all computed by the CPU oracle)."""
from __future__ import annotations

import numpy as np

PADVAL = -9923.0  # the tester's guard value (pdludriver.f:77-79)
NEAR_TIE_REL = 1e-10  # columns whose top-2 |candidates| differ by less are logged
RESID_THRESH = 16.0   # scaled-residual bar for every FP64 run


def system(orc, n, nrhs, kind=1, seed_a=100, seed_b=200, m=None):
    m = n if m is None else m
    A = orc.matgen(m, n, seed_a, kind=kind)
    B = orc.matgen(m, nrhs, seed_b, kind=kind) if nrhs else None
    return A, B


def compare_ipiv(orc, A0, gpu_ipiv_rel, nb, max_replays=4):
    """Compare GPU pivots (1-based, relative to sub(A)) with the oracle's.

    Columns where the oracle's two largest candidates differ by less than
    NEAR_TIE_REL (relative) are logged; a mismatch there is replayed by forcing
    the GPU's pivot in the oracle, so the comparison continues past the tie.
    Returns (n_mismatch_outside_ties, logged_tie_columns).
    """
    m, n = A0.shape
    mn = min(m, n)
    g = np.asarray(gpu_ipiv_rel[:mn], dtype=np.int32)
    force = np.zeros(mn, dtype=np.int32)
    logged = []
    for _ in range(max_replays + 1):
        rec = orc.Recorder(mn, force=force if force.any() else None)
        A = np.asfortranarray(A0.copy())
        with rec:
            ip, _ = orc.pdgetrf(m, n, A, nb=nb)
        ip = ip[:mn]
        ties = set(rec.near_ties(NEAR_TIE_REL).tolist())
        bad = np.nonzero(ip != g)[0]
        if bad.size == 0:
            return 0, sorted(set(logged) | (ties & set(np.nonzero(force)[0].tolist())))
        k = int(bad[0])
        if k in ties:
            logged.append(k)
            force[k] = g[k]
            continue
        return int(bad.size), sorted(set(logged))
    return int(np.count_nonzero(ip != g)), sorted(set(logged))


def padded(a, pad_rows=3, pad_cols=2, ia=1, ja=1):
    """Embed `a` at (ia, ja) of a larger Fortran array filled with PADVAL."""
    m, n = a.shape
    big = np.full((ia - 1 + m + pad_rows, ja - 1 + n + pad_cols), PADVAL, order="F")
    big[ia - 1:ia - 1 + m, ja - 1:ja - 1 + n] = a
    return big


def guards_intact(big, ia, ja, m, n):
    mask = np.ones(big.shape, dtype=bool)
    mask[ia - 1:ia - 1 + m, ja - 1:ja - 1 + n] = False
    return bool(np.all(big[mask] == PADVAL))


def run_pdgesv(sl, ctx, A0, B0, nb, ia=1, ja=1):
    n, nrhs = A0.shape[0], B0.shape[1]
    Ab = padded(A0, ia=ia, ja=ja)
    Bb = padded(B0, ia=ia, ja=1)
    desca = np.array([1, ctx, Ab.shape[0], Ab.shape[1], nb, nb, 0, 0, Ab.shape[0]], np.int32)
    descb = np.array([1, ctx, Bb.shape[0], Bb.shape[1], nb, nb, 0, 0, Bb.shape[0]], np.int32)
    ipiv = np.full(Ab.shape[0] + nb + 4, -77, dtype=np.int32)
    info = sl.pdgesv(n, nrhs, Ab, ia, ja, desca, ipiv, Bb, ia, 1, descb)
    assert guards_intact(Ab, ia, ja, n, n)
    assert guards_intact(Bb, ia, 1, n, nrhs)
    # IPIV entries outside IPIV(IA:IA+N-1) are untouched
    assert np.all(ipiv[:ia - 1] == -77) and np.all(ipiv[ia - 1 + n:] == -77)
    LU = Ab[ia - 1:ia - 1 + n, ja - 1:ja - 1 + n]
    X = Bb[ia - 1:ia - 1 + n, :nrhs]
    rel = ipiv[ia - 1:ia - 1 + n] - (ia - 1)
    return info, np.asfortranarray(LU), rel, np.asfortranarray(X)
