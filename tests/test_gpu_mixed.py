"""GPU tests of the mixed-precision pieces through the C ABI.

The low-precision trailing update C -= L U (BF16/FP16 operands, U scaled per
column by a power of two, FP32 accumulation on tcgen05) is compared with an
FP64 torch reference that applies the same 16-bit rounding and scaling; the
only difference left is FP32 accumulation, bounded by k * 2^-23 relative to
|L| |U|.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref_update(torch, C, L, U, fmt):
    mx = U.abs().amax(dim=0)
    e = torch.where(mx > 0, torch.frexp(mx)[1], torch.zeros_like(mx, dtype=torch.int32))
    Usc = U * torch.ldexp(torch.ones_like(mx), -e)
    scale = torch.ldexp(torch.ones_like(mx, dtype=torch.float64), e.int())
    if fmt == 2:  # BF16x3: hi*hi + hi*lo + lo*hi
        def split(x):
            hi = x.to(torch.bfloat16).float()
            return hi.double(), (x - hi).to(torch.bfloat16).double()
        Lh, Ll = split(L)
        Uh, Ul = split(Usc)
        prod = Lh @ Uh + Lh @ Ul + Ll @ Uh
        bound = Lh.abs() @ Uh.abs() + Lh.abs() @ Ul.abs() + Ll.abs() @ Uh.abs()
        return C.double() - prod * scale, bound * scale
    dt = torch.bfloat16 if fmt == 0 else torch.float16
    Us = Usc.to(dt).double()
    L16 = L.to(dt).double()
    prod = (L16 @ Us) * scale
    bound = (L16.abs() @ Us.abs()) * scale
    return C.double() - prod, bound


@pytest.mark.parametrize("fmt", [0, 1, 2])
@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (1000, 700, 256), (300, 20, 100), (4096, 4096, 256),
                                   (129, 257, 512), (7, 3, 16)])
def test_lowp_update_matches_reference(sl, gpu_required, fmt, m, n, k):
    import torch

    g = torch.Generator(device="cuda").manual_seed(m * 7 + n * 3 + k)
    # column-major FP32 storage: torch tensors of shape (cols, rows)
    Lt = (torch.rand((k, m), device="cuda", generator=g) - 0.5)
    Ut = (torch.rand((n, k), device="cuda", generator=g) - 0.5) * 40.0
    Ct = (torch.rand((n, m), device="cuda", generator=g) - 0.5)
    L, U, C0 = Lt.T, Ut.T, Ct.T.clone()
    ref, bound = _ref_update(torch, C0, L.float(), U.float(), fmt)
    torch.cuda.synchronize()
    info = sl.lib().sl1x1_lowp_update_dev(fmt, m, n, k, Lt.data_ptr(), m, Ut.data_ptr(), k,
                                          Ct.data_ptr(), m, None)
    assert info == 0
    got = Ct.T.double()
    err = (got - ref).abs()
    tol = 4.0 * k * 2.0 ** -23 * bound + 2.0 ** -22 * ref.abs() + 1e-30
    assert bool((err <= tol).all()), float((err / tol).max())


@pytest.mark.parametrize("stages", [2, 3])
@pytest.mark.parametrize("pad", [0, 1, 4])
@pytest.mark.parametrize("fmt,m,n,k", [(2, 1000, 700, 256), (0, 129, 257, 512), (1, 300, 520, 64)])
def test_lowp_update_stages_and_leading_dimension(sl, gpu_required, stages, pad, fmt, m, n, k):
    """Both pipeline depths, and both epilogues: the TMA reduce into C (16-byte
    aligned C, ldc a multiple of 4) and the load/store fallback (pad 1); rows
    between m and ldc must stay untouched."""
    import torch

    ldc = m + pad
    g = torch.Generator(device="cuda").manual_seed(m + 11 * n + k + pad)
    Lt = (torch.rand((k, m), device="cuda", generator=g) - 0.5)
    Ut = (torch.rand((n, k), device="cuda", generator=g) - 0.5) * 3.0
    Cfull = (torch.rand((n, ldc), device="cuda", generator=g) - 0.5)
    C0 = Cfull[:, :m].T.clone()
    guard = Cfull[:, m:].clone()
    ref, bound = _ref_update(torch, C0, Lt.T.float(), Ut.T.float(), fmt)
    L = sl.lib()
    L.sl1x1_set_lowp_stages(stages)
    try:
        torch.cuda.synchronize()
        info = L.sl1x1_lowp_update_dev(fmt, m, n, k, Lt.data_ptr(), m, Ut.data_ptr(), k,
                                       Cfull.data_ptr(), ldc, None)
        torch.cuda.synchronize()
    finally:
        L.sl1x1_set_lowp_stages(2)  # the default
    assert info == 0
    got = Cfull[:, :m].T.double()
    err = (got - ref).abs()
    tol = 4.0 * k * 2.0 ** -23 * bound + 2.0 ** -22 * ref.abs() + 1e-30
    assert bool((err <= tol).all()), float((err / tol).max())
    assert torch.equal(Cfull[:, m:], guard)


def _dev_colmajor(torch, M):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(M).T)).cuda()


def _solve_ir(sl, torch, A0, B0, fmt, tol=1.0, nb=256):
    n, nrhs = A0.shape[0], B0.shape[1]
    dA = _dev_colmajor(torch, A0)
    dB = _dev_colmajor(torch, B0)
    dX = torch.zeros_like(dB)
    dpiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    info, it, st = sl.dgesv_ir_dev(n, nrhs, dA.data_ptr(), n, dpiv.data_ptr(), dB.data_ptr(), n,
                                   dX.data_ptr(), n, fmt=fmt, nb=nb, tol=tol, keep_a=True)
    A_after = dA.cpu().numpy().T
    return info, it, st, np.asfortranarray(dX.cpu().numpy().T), A_after


@pytest.fixture
def no_cost_rule(sl):
    """Refinement without the cost rule (it stops only on a stall), for tests
    of what the refinement itself reaches."""
    sl.lib().sl1x1_set_ir_cost_ratio(0.0)
    yield
    sl.lib().sl1x1_set_ir_cost_ratio(3.5)


@pytest.mark.parametrize("fmt", ["bf16", "fp16", "bf16x3"])
@pytest.mark.parametrize("n,nrhs,nb", [(64, 1, 32), (1000, 2, 256), (2500, 1, 256), (700, 3, 128)])
def test_mixed_ir_reaches_fp64_backward_error(sl, orc, gpu_required, no_cost_rule, fmt, n, nrhs, nb):
    import torch
    from lu_helpers import system

    A0, B0 = system(orc, n, nrhs)
    info, it, st, X, A_after = _solve_ir(sl, torch, A0, B0, fmt, nb=nb)
    assert info == 0
    np.testing.assert_array_equal(A_after, A0)  # keep_a: A untouched
    sr = orc.sresid(A0, B0, X)  # the FP64 oracle's scaled residual
    assert sr < 16.0
    assert st["sresid"] <= 1.0 + 1e-9 or st["fell_back"] == 1
    assert st["fell_back"] == 0, st
    assert it >= 0


@pytest.mark.parametrize("kappa", [1e2, 1e4, 1e6, 1e8])
def test_mixed_ir_conditioning_sweep(sl, orc, gpu_required, no_cost_rule, kappa):
    # A = U diag(s) V^T with seeded Householder reflectors, s geometric 1 -> 1/kappa
    import torch

    n, nrhs = 384, 4
    A0 = orc.gen_conditioned(n, kappa, nrefl=16, seed=1000)
    B0 = orc.matgen(n, nrhs, 200, kind=0)  # uniform (-1, 1]
    for fmt in ("bf16", "bf16x3"):
        info, it, st, X, _ = _solve_ir(sl, torch, A0, B0, fmt, nb=64)
        assert info == 0
        assert orc.sresid(A0, B0, X) < 16.0  # refinement or the FP64 fallback, never worse
        if kappa <= 1e2 or (fmt == "bf16x3" and kappa <= 1e4):
            assert st["fell_back"] == 0, (fmt, st)


def test_gmres_ir_converges_at_kappa_1e8_without_fallback(sl, orc, gpu_required, no_cost_rule):
    # kappa = 1e8 is beyond classical refinement with BF16x3 (near-FP32) factors;
    # GMRES-IR applies the preconditioner (FP32 factors and block inverses) with
    # FP64 vector arithmetic, a fixed operator, and reaches the FP64 backward error
    # without falling back to the FP64 factorization.
    import torch

    n, nrhs = 1024, 4
    A0 = orc.gen_conditioned(n, 1e8, nrefl=64, seed=1000)
    B0 = orc.matgen(n, nrhs, 200, kind=0)
    info, it, st, X, _ = _solve_ir(sl, torch, A0, B0, "bf16x3", nb=64)
    assert info == 0
    assert st["fell_back"] == 0, st
    assert st["gmres_outer"] >= 1, st
    assert st["sresid"] <= 1.0 + 1e-9, st
    assert orc.sresid(A0, B0, X) < 16.0


def test_mixed_ir_singular_falls_back_and_reports_info(sl, orc, gpu_required):
    import torch
    from lu_helpers import system

    n = 200
    A0, B0 = system(orc, n, 1)
    A0[:, 17] = 0.0
    info, it, st, X, _ = _solve_ir(sl, torch, A0, B0, "bf16", nb=64)
    assert info == 18
    assert st["fell_back"] == 1 and it == -1


def test_cost_rule_falls_back_early_and_stays_correct(sl, orc, gpu_required):
    """BF16 factors of a kappa = 1e8 matrix: GMRES-IR would need many
    iterations; with the cost rule on (a small ratio, so that any slow
    convergence counts) refinement gives up within its first cycle, reports
    fell_back = 2 and the FP64 solve gives the FP64 backward error."""
    import torch

    n, nrhs = 1024, 2
    A0 = orc.gen_conditioned(n, 1e8, nrefl=64, seed=1000)
    B0 = orc.matgen(n, nrhs, 200, kind=0)
    L = sl.lib()
    L.sl1x1_set_ir_cost_ratio(0.5)
    try:
        info, it, st, X, _ = _solve_ir(sl, torch, A0, B0, "bf16", nb=64)
    finally:
        L.sl1x1_set_ir_cost_ratio(3.5)
    assert info == 0
    assert st["fell_back"] == 2, st
    assert it == -3
    assert st["gmres_inner"] < 100, st
    assert orc.sresid(A0, B0, X) < 16.0
