"""GPU tests of the sliced FP64 product on the BF16 tensor cores
(sl1x1_ozgemm_dev, the trailing update of the plain LU):

* bit-exact against exact rational arithmetic on inputs whose slices stop at
  the third (so every diagonal of slice products is summed exactly), including
  operands at full slice magnitude, where the sums reach 3 * 256 * 127^2 —
  the tensor core's FP32 accumulation must not lose a unit;
* on general FP64 data, the error against a 113-bit (quad) or 64-bit
  (x87) product is within a few units of 2^-53 of max|A(i,:)| max|B(:,j)|,
  no worse than FP64 DMMA's on the same product;
* K above 256 runs in passes; Inf and NaN poison their row or column;
* the LU with the sliced update gives the same pivots as with the DMMA one
  and the same scaled residuals bar;
* the power-of-two balancing along k keeps row-graded operands (an LU step
  whose pivots span 2^+-20 .. 2^+-300) at componentwise FP64 accuracy, and
  operands outside the error budget take the FP64 route (counted by
  sl1x1_ozgemm_fp64_routes), pass by pass, with C aliasing B allowed.
"""
import math
from fractions import Fraction

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_dev(sl, gpu_required):
    import torch

    assert sl.lib().sl1x1_device_ok() == 1
    return torch, torch.device("cuda", 0)


def run_oz(sl, torch, dev, A, B, C, alpha=-1.0):
    m, k = A.shape
    n = B.shape[1]
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)  # column-major: store A^T row-major
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).to(dev)
    dC = torch.from_numpy(np.ascontiguousarray(C.T)).to(dev)
    rc = sl.ozgemm_dev(m, n, k, alpha, dA.data_ptr(), m, dB.data_ptr(), k, dC.data_ptr(), m)
    assert rc == 0
    torch.cuda.synchronize()
    return dC.cpu().numpy().T.copy()


def exact_update(A, B, C, alpha):
    """The sliced product's result for operands whose row / column slices are
    all exact (<= 21 bits below each scale): one pass per 256 columns of K,
    I = 2^52 (A B)_ij / 2^(e_i + f_j) rounded once to FP64, then one FMA,
    with e_i, f_j the balanced scale exponents (tests/oz_model.py)."""
    from oz_model import scales

    m, k = A.shape
    n = B.shape[1]
    out = C.copy()
    for k0 in range(0, k, 256):
        Ak, Bk = A[:, k0:k0 + 256], B[k0:k0 + 256, :]
        e, f, tripped, _ = scales(Ak, Bk)
        assert not tripped
        e = [0 if v is None else v for v in e]
        f = [0 if v is None else v for v in f]
        Af = [[Fraction(float(x)) for x in Ak[i]] for i in range(m)]
        Bf = [[Fraction(float(x)) for x in Bk[:, j]] for j in range(n)]
        for i in range(m):
            for j in range(n):
                dot = sum(a * b for a, b in zip(Af[i], Bf[j]))
                I = dot * Fraction(2) ** (52 - e[i] - f[j])
                assert I.denominator == 1
                Id = float(int(I))  # round-to-nearest-even, as the device conversion
                scale = Fraction(alpha) * Fraction(2) ** (e[i] + f[j] - 52)
                out[i, j] = float(Fraction(float(out[i, j])) + scale * Fraction(Id))
    return out


def short_operands(rng, rows, cols, bits=21, full=False, axis=1):
    """Entries u * 2^(ex - bits) with |u| < 2^bits, per-row (axis=1) or
    per-column exponents ex; full=True puts every slice at +-127."""
    if full:
        u = np.full((rows, cols), float(2 ** bits - 1))
    else:
        u = rng.integers(-(2 ** bits) + 1, 2 ** bits, size=(rows, cols)).astype(np.float64)
    ex = rng.integers(-6, 7, size=rows if axis == 1 else cols)
    scale = np.exp2(ex - bits)
    return u * (scale[:, None] if axis == 1 else scale[None, :])


@pytest.mark.parametrize("m,n,k,full", [(37, 29, 256, True), (37, 29, 256, False),
                                        (130, 70, 100, False), (20, 9, 300, False)])
def test_bit_exact_on_exact_slices(sl, torch_dev, m, n, k, full):
    torch, dev = torch_dev
    rng = np.random.default_rng(m * 1000 + n + k)
    A = short_operands(rng, m, k, full=full, axis=1)
    B = short_operands(rng, k, n, full=full, axis=0)
    if full:  # one sign everywhere: the largest sums the accumulators can see
        A, B = np.abs(A), np.abs(B)
    C = rng.uniform(-1, 1, (m, n))
    got = run_oz(sl, torch, dev, A, B, C, alpha=-1.0)
    want = exact_update(A, B, C, -1.0)
    np.testing.assert_array_equal(got, want)


def _wide(a):
    return a.astype(np.longdouble)


@pytest.mark.parametrize("m,n,k", [(300, 200, 256), (257, 65, 64), (128, 64, 512)])
def test_error_within_fp64_bound(sl, torch_dev, m, n, k):
    torch, dev = torch_dev
    rng = np.random.default_rng(7 + m + n + k)
    A = rng.uniform(-0.5, 0.5, (m, k)) * np.exp2(rng.integers(-3, 4, size=(m, 1)))
    B = rng.uniform(-0.5, 0.5, (k, n))
    C = rng.uniform(-1, 1, (m, n))
    got = run_oz(sl, torch, dev, A, B, C, alpha=-1.0)
    ref = _wide(C) - _wide(A) @ _wide(B)
    # scale of each entry: per-pass row max x column max x K
    scl = np.zeros((m, n))
    for k0 in range(0, k, 256):
        ra = np.max(np.abs(A[:, k0:k0 + 256]), axis=1)
        cb = np.max(np.abs(B[k0:k0 + 256, :]), axis=0)
        scl += np.outer(ra, cb)
    err = np.abs((got.astype(np.longdouble) - ref).astype(np.float64))
    eps = 2.0 ** -53
    # dropped slice products (d >= 10): about 2^-52 of the scales per entry,
    # at most 2^-44.8; the final rounding adds half a unit of |C|
    assert np.max(err / (scl * eps + np.abs(ref.astype(np.float64)) * eps)) < 256.0
    # no worse than an FP64 GEMM (host BLAS) on the same product
    ref64 = C - A @ B
    err64 = np.abs((ref64.astype(np.longdouble) - ref).astype(np.float64))
    assert np.linalg.norm(err) <= 2.0 * np.linalg.norm(err64) + 1e-300


def test_nonfinite_rows_and_columns(sl, torch_dev):
    torch, dev = torch_dev
    rng = np.random.default_rng(11)
    m, n, k = 50, 40, 64
    A = rng.uniform(-1, 1, (m, k))
    B = rng.uniform(-1, 1, (k, n))
    A[3, 5] = np.nan
    B[7, 9] = np.inf
    C = rng.uniform(-1, 1, (m, n))
    got = run_oz(sl, torch, dev, A, B, C)
    assert np.all(np.isnan(got[3, :]))
    assert np.all(np.isnan(got[:, 9]))
    mask = np.ones((m, n), bool)
    mask[3, :] = False
    mask[:, 9] = False
    ref = C - A @ B
    assert np.all(np.isfinite(got[mask]))
    assert np.max(np.abs(got[mask] - ref[mask])) < 1e-13


def test_zero_rows_and_empty(sl, torch_dev):
    torch, dev = torch_dev
    rng = np.random.default_rng(12)
    m, n, k = 70, 33, 40
    A = rng.uniform(-1, 1, (m, k))
    A[10, :] = 0.0
    B = rng.uniform(-1, 1, (k, n))
    B[:, 4] = 0.0
    C = rng.uniform(-1, 1, (m, n))
    got = run_oz(sl, torch, dev, A, B, C)
    np.testing.assert_array_equal(got[10, :], C[10, :])
    np.testing.assert_array_equal(got[:, 4], C[:, 4])
    assert sl.ozgemm_dev(0, 5, 5, 1.0, 0, 1, 0, 5, 0, 1) == 0
    assert sl.ozgemm_dev(-1, 5, 5, 1.0, 0, 1, 0, 5, 0, 1) == -1


@pytest.mark.parametrize("n,nb", [(1000, 256), (777, 128), (600, 320)])
def test_lu_sliced_update_matches_dmma_pivots(sl, orc, torch_dev, n, nb):
    torch, dev = torch_dev
    rng = np.random.default_rng(n + nb)
    A = rng.uniform(-0.5, 0.5, (n, n))
    res = {}
    try:
        for mode in (0, 1):
            sl.set_f64_update(mode)
            dA = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)
            piv = torch.zeros(n, dtype=torch.int32, device=dev)
            assert sl.dgetrf_dev(n, n, dA.data_ptr(), n, piv.data_ptr(), nb) == 0
            res[mode] = (dA.cpu().numpy().T.copy(), piv.cpu().numpy().copy())
    finally:
        sl.set_f64_update(1)
    np.testing.assert_array_equal(res[0][1], res[1][1])
    for mode in (0, 1):
        LU, piv = res[mode]
        assert orc.fresid(LU, piv, A) < 16.0
    # the two factorizations agree to rounding
    assert np.max(np.abs(res[0][0] - res[1][0])) < 1e-10


def test_tiles_per_cta_changes_only_speed(sl, torch_dev):
    # every tile's products and epilogue are the same whichever CTA runs it
    torch, dev = torch_dev
    rng = np.random.default_rng(21)
    m, n, k = 700, 500, 256
    A = rng.uniform(-1, 1, (m, k))
    B = rng.uniform(-1, 1, (k, n))
    C = rng.uniform(-1, 1, (m, n))
    L = sl.lib()
    outs = []
    try:
        for t in (1, 4, 16):
            L.sl1x1_set_ozgemm_tiles(t)
            outs.append(run_oz(sl, torch, dev, A, B, C))
    finally:
        L.sl1x1_set_ozgemm_tiles(4)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])


def _routes(sl):
    r = sl.lib().sl1x1_ozgemm_fp64_routes()
    assert r >= 0
    return r


def _componentwise_ok(got, A, B, C, alpha, c):
    """|got - exact| <= c K eps (|A||B|)_ij + 2 eps |exact|, exact in wide
    arithmetic; returns the worst ratio to that bound."""
    ref = _wide(C) + alpha * (_wide(A) @ _wide(B))
    absab = np.abs(A) @ np.abs(B)
    k = A.shape[1]
    eps = 2.0 ** -53
    err = np.abs((got.astype(np.longdouble) - ref).astype(np.float64))
    tol = c * k * eps * absab + 2 * eps * np.abs(ref.astype(np.float64)) + 1e-300
    return float(np.max(err / tol))


@pytest.mark.parametrize("spread", [20, 60, 300])
def test_row_graded_operands_componentwise(sl, torch_dev, spread):
    """L21 / U12 of a row-graded LU step (pivots spanning 2^+-spread inside one
    block): the balancing keeps every entry within a few units of 2^-53 of
    its own |A||B| (without it the error scale would exceed the terms by
    more than the spread, in bits), and no pass takes the FP64 route."""
    from oz_model import graded_lu_operands, scales

    torch, dev = torch_dev
    rng = np.random.default_rng(spread)
    m, k, n = 300, 256, 200
    A, B = graded_lu_operands(rng, m, k, n, spread)
    assert not scales(A, B)[2]
    C = (np.abs(A) @ np.abs(B)) * rng.uniform(-1, 1, (m, n))
    r0 = _routes(sl)
    got = run_oz(sl, torch, dev, A, B, C, alpha=-1.0)
    assert _routes(sl) == r0
    assert _componentwise_ok(got, A, B, C, -1.0, c=2.0) <= 1.0


@pytest.mark.parametrize("spread", [0, 40])
def test_column_and_row_scaled_operands(sl, torch_dev, spread):
    """Operands scaled by powers of two on both sides (D1 A D2, D2^-1 B D3):
    the result is that of the unscaled product to componentwise accuracy."""
    torch, dev = torch_dev
    rng = np.random.default_rng(100 + spread)
    m, k, n = 257, 190, 130
    d = np.exp2(rng.integers(-spread, spread + 1, size=k))
    A = rng.uniform(-1, 1, (m, k)) * d[None, :]
    A *= np.exp2(rng.integers(-spread, spread + 1, size=(m, 1)))
    B = rng.uniform(-1, 1, (k, n)) / d[:, None]
    B *= np.exp2(rng.integers(-spread, spread + 1, size=(1, n)))
    C = np.zeros((m, n))
    r0 = _routes(sl)
    got = run_oz(sl, torch, dev, A, B, C, alpha=1.0)
    assert _routes(sl) == r0
    assert _componentwise_ok(got, A, B, C, 1.0, c=2.0) <= 1.0


def test_spike_operands_take_fp64_route(sl, torch_dev):
    """A row of B with one entry 2^40 above the rest, met by a 2^-50 entry of
    A: the row budget test trips, the pass runs in FP64 arithmetic, and every
    entry is within the FP64 GEMM's componentwise bound."""
    from oz_model import scales, spike_operands

    torch, dev = torch_dev
    rng = np.random.default_rng(31)
    m, k, n = 300, 200, 150
    A, B = spike_operands(rng, m, k, n)
    assert scales(A, B)[2]
    C = rng.uniform(-1, 1, (m, n))
    r0 = _routes(sl)
    got = run_oz(sl, torch, dev, A, B, C, alpha=-1.0)
    assert _routes(sl) == r0 + 1
    assert _componentwise_ok(got, A, B, C, -1.0, c=1.0) <= 1.0
    # the next product is sliced again: the route flag belongs to its pass
    A2 = rng.uniform(-1, 1, (m, k))
    B2 = rng.uniform(-1, 1, (k, n))
    got2 = run_oz(sl, torch, dev, A2, B2, C, alpha=-1.0)
    assert _routes(sl) == r0 + 1
    assert _componentwise_ok(got2, A2, B2, C, -1.0, c=4.0) <= 1.0


def test_fp64_route_per_pass_of_k(sl, torch_dev):
    """K = 300 runs in two passes; only the second is outside the budget."""
    from oz_model import spike_operands

    torch, dev = torch_dev
    rng = np.random.default_rng(32)
    m, n = 200, 100
    A1 = rng.uniform(-1, 1, (m, 256))
    B1 = rng.uniform(-1, 1, (256, n))
    A2, B2 = spike_operands(rng, m, 44, n)
    A = np.hstack([A1, A2])
    B = np.vstack([B1, B2])
    C = rng.uniform(-1, 1, (m, n))
    r0 = _routes(sl)
    got = run_oz(sl, torch, dev, A, B, C, alpha=-1.0)
    assert _routes(sl) == r0 + 1
    assert _componentwise_ok(got, A, B, C, -1.0, c=4.0) <= 1.0


@pytest.mark.parametrize("k", [64, 256])
def test_fp64_route_with_c_aliasing_b(sl, torch_dev, k):
    """The U12 solve's form C = B (m = k, up to 256 rows: two row tiles): on
    the FP64 route each CTA takes whole column blocks and reads its columns
    of B before writing them."""
    from oz_model import spike_operands

    torch, dev = torch_dev
    rng = np.random.default_rng(33 + k)
    n = 300
    A, B = spike_operands(rng, k, k, n)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).to(dev)
    r0 = _routes(sl)
    rc = sl.ozgemm_dev(k, n, k, 1.0, dA.data_ptr(), k, dB.data_ptr(), k, dB.data_ptr(), k)
    assert rc == 0
    torch.cuda.synchronize()
    assert _routes(sl) == r0 + 1
    got = dB.cpu().numpy().T
    assert _componentwise_ok(got, A, B, B, 1.0, c=1.0) <= 1.0
