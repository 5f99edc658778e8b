"""CPU checks of the arithmetic behind the sliced FP64 product (the trailing
update of the plain LU, scalapack_gb300/csrc/ozgemm_f64.cu), restated here in
numpy and exact Python integers:

* the integer split of an FP64 value -- significand shifted into a 56-bit
  fixed point relative to the row scale 2^e, 7-bit fields with the sign --
  equals the FP64 truncation x 2^-e = sum_s a_s 2^-7s (|a_s| <= 127), and the
  eight slices reproduce x to within one unit of 2^(e-56);
* every slice is exactly representable in BF16 (8 significant bits) after its
  2^-7(s-1) weight;
* for K <= 256 a diagonal's products stay below 2^24 while it holds at most
  4 of them, which is what makes the FP32 tensor-core sums exact;
* the epilogue's integer I = sum_d P_d 2^(52-7d) fits in 64 bits.
"""
import math
from fractions import Fraction

import numpy as np


def frexp_exp(amax):
    return math.frexp(amax)[1] if amax > 0 else 0


def fixed56(x, e):
    """floor(|x| 2^(56-e)) from the bit pattern, as the device does."""
    bits = np.float64(x).view(np.uint64).item()
    bexp = (bits >> 52) & 0x7FF
    mant = bits & ((1 << 52) - 1)
    if bexp:
        mant |= 1 << 52
        q = bexp - 1075
    else:
        q = -1074
    sh = q - e + 56
    if sh >= 0:
        return mant << sh
    if sh <= -64:
        return 0
    return mant >> (-sh)


def slices(x, e):
    u = fixed56(abs(x), e)
    assert u < (1 << 56)
    a = [(u >> (49 - 7 * s)) & 127 for s in range(8)]
    return [-v if x < 0 else v for v in a]


def trunc_slices(x, e):
    """The FP64 truncation recurrence the kernel's comment states."""
    y = Fraction(x) / Fraction(2) ** e * 128
    out = []
    for _ in range(8):
        a = int(y)  # truncation toward zero
        out.append(a)
        y = (y - a) * 128
    return out


def test_integer_split_equals_truncation_and_reconstructs():
    rng = np.random.default_rng(5)
    rows = [rng.uniform(-1, 1, 64) * 2.0 ** rng.integers(-30, 30),
            rng.standard_normal(64) * 1e-300,         # tiny, subnormal neighbours
            np.array([5e-324, -5e-324, 1e-310, 0.0, 2.0 ** -1022, 1.0]),
            rng.uniform(-1, 1, 64) * 1e300]
    for row in rows:
        e = frexp_exp(float(np.max(np.abs(row))))
        for x in row:
            x = float(x)
            a = slices(x, e)
            assert a == trunc_slices(x, e), (x, e)
            assert all(abs(v) <= 127 for v in a)
            rec = sum(Fraction(v) * Fraction(2) ** (e - 7 * (s + 1)) for s, v in enumerate(a))
            err = abs(Fraction(x) - rec)
            assert err < Fraction(2) ** (e - 56), (x, float(err))


def test_weighted_slices_are_exact_bf16():
    # a_s 2^-7(s-1) with |a_s| <= 127: 8 significant bits at most, exponent in range
    for s in range(8):
        for a in (1, 3, 5, 64, 85, 127, -127, -1):
            v = np.float32(a) * np.float32(2.0 ** (-7 * s))
            bits = np.array([v], dtype=np.float32).view(np.uint32)[0]
            assert (int(bits) & 0xFFFF) == 0  # the low 16 bits are zero: BF16 holds it exactly


def test_diagonal_sums_within_fp32_exact_range():
    kmax = 256
    one = kmax * 127 * 127
    assert one < 2 ** 22
    for products in (1, 2, 3, 4):
        assert products * one < 2 ** 24  # d <= 5 hold at most 4 products: exact
    assert 5 * one >= 2 ** 24 > 4 * one  # d = 6 is exact unless nearly every term is extreme


def test_combined_integer_fits_int64():
    one = 256 * 127 * 127
    worst = (one << 38) + (2 * one << 31) + (3 * one << 24) + (4 * one << 17) + (5 * one << 10)
    tail = int(6 * one * 8 * 1.01)  # P7 plus the scaled P8, P9, with 3 fraction bits
    assert worst + tail < 2 ** 63
    # and the conversion to FP64 rounds once: the value has at most 61 significant bits
    assert (worst + tail).bit_length() <= 62


# ---- balancing along k and the error budget (tests/oz_model.py) ----------

def test_balancing_removes_the_pivot_spread_of_a_graded_step():
    """Row-graded LU step: without the balancing the error scale 2^(e_i+f_j)
    exceeds the largest term of some entry by more than the spread of the
    block's pivots (in bits); with it, by a couple of bits, and the pass stays
    inside the budget."""
    import oz_model as M

    rng = np.random.default_rng(3)
    for spread in (20, 60, 300):
        A, B = M.graded_lu_operands(rng, 120, 64, 90, spread)
        assert M.bound_gap_bits(A, B, balance=False) > spread
        assert M.bound_gap_bits(A, B) < 3.0
        assert not M.scales(A, B)[2]


def test_side_b_for_the_graded_inverse_product():
    """(inv(L_bb) - I) A12_b on a graded block: balancing by A's columns
    leaves rows whose terms sit far below their scale (the budget trips),
    balancing by B's rows lines every term up."""
    import oz_model as M

    rng = np.random.default_rng(7)
    A, B = M.graded_inverse_operands(rng, 64, 80, 60)
    assert M.scales(A, B, side="A")[2]
    assert not M.scales(A, B, side="B")[2]
    # entrywise, side B's error scale sits about the pivots' spread closer
    # to the terms than side A's
    assert M.bound_gap_bits(A, B, side="B") < M.bound_gap_bits(A, B, side="A") - 20


def test_budget_passes_well_scaled_and_diagonally_scaled_operands():
    import oz_model as M

    rng = np.random.default_rng(4)
    A = rng.uniform(-0.5, 0.5, (300, 256))
    B = rng.uniform(-0.5, 0.5, (256, 200)) * 40
    assert not M.scales(A, B)[2]
    d = np.exp2(rng.integers(-200, 200, size=256))
    assert not M.scales(A / d[None, :], B * d[:, None])[2]  # any scaling along k
    r = np.exp2(rng.integers(-200, 200, size=300))
    c = np.exp2(rng.integers(-200, 200, size=200))
    assert not M.scales(A * r[:, None], B * c[None, :])[2]


def test_budget_trips_where_no_balancing_helps():
    """A row of B with one entry 2^40 above the rest, met by a 2^-50 entry of
    A: row 0's largest term needs the k = 0 product in full, but row 0's
    scale is set by the other k, so the slices keep only 6 of its bits."""
    import oz_model as M

    rng = np.random.default_rng(5)
    A, B = M.spike_operands(rng, 60, 32, 40)
    e, f, tripped, info = M.scales(A, B)
    assert tripped
    assert info["gap"][0] > 30
    big = np.abs(A[:, 0]) >= 0.5  # rows whose k = 0 entry is near column 0's maximum pass
    assert np.all(info["gap"][big] <= M.BUDGET)
    assert M.bound_gap_bits(A, B) > 30


def test_budget_trips_when_a_scale_leaves_the_normal_range():
    import oz_model as M

    rng = np.random.default_rng(6)
    A = rng.uniform(-1, 1, (10, 8)) * 2.0 ** -1000
    B = rng.uniform(-1, 1, (8, 6))
    assert M.scales(A, B)[2]  # e_i - 26 below the normal range
    assert not M.scales(A * 2.0 ** 1000, B)[2]
