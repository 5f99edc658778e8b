"""Shared helpers for the GPU parity tests: inputs from the tester's generator,
the IPIV comparison with near-tie logging and forced-pivot replay, and the
tester's scaled residuals (all computed by the CPU oracle)."""
from __future__ import annotations

import numpy as np

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
