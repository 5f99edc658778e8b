"""GPU parity of the default (sliced-product) FP64 path on badly scaled
inputs, through pdgesv_: IPIV identical to the oracle's outside logged near
ties, both scaled residuals below 16, and the number of sliced-product passes
that took the FP64 route.

The sliced product keeps 56 bits below each row's and column's scale after
an exact power-of-two balancing along k (scalapack_gb300/csrc/ozgemm_f64.cu).
Row and column scalings of any size (2^+-60, 2^+-300), one dominant entry per
row and the tester's diagonally dominant form (TESTING/traditional/LIN/
pdmatgen.f:515-542) stay on the tensor cores; a matrix whose update needs
the product of a tiny L entry and a huge U entry at full precision trips the
error budget and that product is computed in FP64 by the same launches.
"""
import numpy as np
import pytest

from lu_helpers import RESID_THRESH, compare_ipiv, run_pdgesv

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(sl, gpu_required):
    assert sl.lib().sl1x1_device_ok() == 1
    return sl.blacs_gridinit(1, 1)


def _routes(sl):
    r = sl.lib().sl1x1_ozgemm_fp64_routes()
    assert r >= 0
    return r


def graded(orc, n, kind, seed=100):
    """Test matrices: base = the tester's generator on U[-0.5, 0.5]."""
    rng = np.random.default_rng(seed + n)
    A = np.asfortranarray(orc.matgen(n, n, seed, kind=1))
    if kind == "rows60":
        A *= np.exp2(rng.integers(-60, 61, size=(n, 1)))
    elif kind == "cols60":
        A *= np.exp2(rng.integers(-60, 61, size=(1, n)))
    elif kind == "both300":
        A *= np.exp2(rng.integers(-150, 151, size=(n, 1)))
        A *= np.exp2(rng.integers(-150, 151, size=(1, n)))
    elif kind == "rows_smooth":  # row i scaled by 2^(-100 i / n): pivots sweep downwards
        A *= np.exp2(np.floor(-100.0 * np.arange(n) / n))[:, None]
    elif kind == "dominant":  # one entry 2^40 per row, in a random column
        perm = rng.permutation(n)
        A[np.arange(n), perm] = np.sign(A[np.arange(n), perm]) * 2.0 ** 40
    elif kind == "diag_d":  # PDMATGEN DIAG='D': |a_ii| + max(M, N) on the diagonal
        A = np.asfortranarray(orc.matgen(n, n, seed, kind=0, diag=True))
    else:
        raise ValueError(kind)
    return np.asfortranarray(A)


@pytest.mark.parametrize("kind", ["rows60", "cols60", "both300", "rows_smooth", "dominant",
                                  "diag_d"])
@pytest.mark.parametrize("n,nb", [(1024, 256), (777, 128)])
def test_badly_scaled_parity(sl, orc, ctx, kind, n, nb):
    A0 = graded(orc, n, kind)
    B0 = np.asfortranarray(orc.matgen(n, 2, 200, kind=1))
    r0 = _routes(sl)
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, nb)
    assert info == 0
    if n == 1024:
        # the balancing keeps every product of these factorizations on the
        # tensor cores (at NB = 128 a product over a subset of the columns can
        # exceed the budget by a bit now and then and take the FP64 route)
        assert _routes(sl) == r0
    bad, ties = compare_ipiv(orc, A0, rel, nb)
    assert bad == 0, f"IPIV differs outside near-ties (ties logged: {ties})"
    assert orc.fresid(LU, rel, A0) < RESID_THRESH
    assert orc.sresid(A0, B0, X) < RESID_THRESH


def spike_matrix(orc, n, nb, j0):
    """A matrix whose first trailing update needs a tiny L entry times a huge
    U entry at full precision:
    * row 3 is column 0's pivot (A[3, 0] = 4);
    * row 7 is zero in the panel's columns except 4 in the last one, so it is
      that column's pivot and row nb-1 of U12 is row 7's trailing part
      unchanged: 2^40 in column j0 (the last row of a forward substitution
      spreads into no other row);
    * row 9 is half of row 3 in the panel plus 2^-30 in its last column, so
      after column 0 its entries cancel exactly: L(9, :) = [0.5, 0, ..., 0,
      ~2^-29], never a pivot.
    Row 9's slices are scaled by its 0.5 at k = 0, while its largest term,
    2^-29 * 2^40, comes from k = nb-1: 28 bits beyond the budget."""
    A = np.asfortranarray(orc.matgen(n, n, 100, kind=1))
    A[3, 0] = 4.0
    A[7, :nb - 1] = 0.0
    A[7, nb - 1] = 4.0
    A[7, j0] = 2.0 ** 40
    A[9, :nb] = 0.5 * A[3, :nb]
    A[9, nb - 1] += 2.0 ** -30
    return A


def test_budget_sends_the_spike_update_to_fp64(sl, orc, ctx):
    n, nb = 600, 128
    A0 = spike_matrix(orc, n, nb, j0=400)
    B0 = np.asfortranarray(orc.matgen(n, 1, 200, kind=1))
    r0 = _routes(sl)
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, nb)
    assert info == 0
    assert _routes(sl) > r0
    bad, ties = compare_ipiv(orc, A0, rel, nb)
    assert bad == 0, f"IPIV differs outside near-ties (ties logged: {ties})"
    assert orc.fresid(LU, rel, A0) < RESID_THRESH
    assert orc.sresid(A0, B0, X) < RESID_THRESH
    # the factors agree with the oracle's relative to each row's scale; the
    # sliced product would have kept 27 bits of row 9's 2^11 term, an error of
    # about 7e-9 of that row's scale
    LUo = np.asfortranarray(A0.copy())
    orc.pdgetrf(n, n, LUo, nb=nb)
    scale = np.max(np.abs(LUo), axis=1, keepdims=True)
    assert np.max(np.abs(LU - LUo) / scale) < 1e-9


@pytest.mark.parametrize("kind", ["rows60", "both300"])
def test_graded_sliced_and_dmma_modes_agree(sl, orc, ctx, kind):
    """The same graded matrix through the FP64 DMMA update: same pivots, and
    factors equal to rounding (amplified by the elimination) relative to each
    row's scale."""
    n, nb = 640, 128
    A0 = graded(orc, n, kind)
    B0 = np.asfortranarray(orc.matgen(n, 1, 200, kind=1))
    out = {}
    try:
        for mode in (0, 1):
            sl.set_f64_update(mode)
            out[mode] = run_pdgesv(sl, ctx, A0, B0, nb)
    finally:
        sl.set_f64_update(1)
    np.testing.assert_array_equal(out[0][2], out[1][2])
    LU0, LU1 = out[0][1], out[1][1]
    scale = np.maximum(np.max(np.abs(LU0), axis=1, keepdims=True), 1e-300)
    assert np.max(np.abs(LU0 - LU1) / scale) < 1e-8
