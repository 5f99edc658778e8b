"""Oracle-checked GPU runs at the full configured sizes of the mixed-precision
and batched forms (the plain FP64 N=16384 case is in test_gpu_lu.py):

* mixed LU-IR at N=32768, NRHS=1, A and B iid U[-0.5,0.5] -- every run, in
  each of the three trailing-update formats, ends with the CPU oracle's FP64
  scaled residual ||b - Ax|| / (||A|| ||x|| N eps) below 16 (refinement, or
  the plain FP64 fallback when refinement stalls);
* the conditioning sweep at N=8192, NRHS=4, A = (H_1..H_64) diag(s)
  (G_1..G_64)^T with s geometric from 1 to 1/kappa, kappa in {1e2, 1e4, 1e6,
  1e8} (the pattern of TOOLS/LAPACK/dlagge.f), B iid U[-1,1];
* all 4096 systems of the batched form (N ~ U{16..512}, NRHS ~ U{1..8},
  U[-0.5,0.5] plus N/4 on the diagonal of half of them), FP64 and FP32-factor +
  FP64-IR plans, each system's residual computed by the oracle, not by the
  kernel.

Inputs are generated on the GPU with torch's seeded generator (the shapes and
distributions the benchmark uses); the residuals come from the oracle's FP64
host arithmetic on copies of A, B and X.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host(t):
    """Column-major host copy of a device tensor holding A^T row-major."""
    return np.asfortranarray(t.cpu().numpy().T)


@pytest.fixture(scope="module")
def mixed_32768(sl, gpu_required):
    import torch

    n = 32768
    g = torch.Generator(device="cuda").manual_seed(2024 + 17)
    At = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=g) - 0.5
    Bt = torch.rand((1, n), dtype=torch.float64, device="cuda", generator=g) - 0.5
    yield n, At, Bt
    del At, Bt
    torch.cuda.empty_cache()


def test_mixed_ir_n32768_every_format_against_oracle(sl, orc, mixed_32768):
    import torch

    n, At, Bt = mixed_32768
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    Xs = {}
    for fmt in ("bf16x3", "fp16", "bf16"):
        Xt = torch.zeros_like(Bt)
        torch.cuda.synchronize()
        info, it, st = sl.dgesv_ir_dev(n, 1, At.data_ptr(), n, piv.data_ptr(), Bt.data_ptr(), n,
                                       Xt.data_ptr(), n, fmt=fmt, nb=256, tol=1.0, keep_a=True)
        assert info == 0, (fmt, st)
        assert st["sresid"] <= 1.0 + 1e-9, (fmt, st)  # the solver's own stopping test
        Xs[fmt] = (_host(Xt), st)
    A = _host(At)
    B = _host(Bt)
    for fmt, (X, st) in Xs.items():
        r = orc.sresid(A, B, X)
        assert r < 16.0, (fmt, r, st)
        # the device residual the solver stopped on agrees with the oracle's
        assert r <= 16.0 * max(st["sresid"], 1e-3), (fmt, r, st["sresid"])
    assert Xs["bf16x3"][1]["fell_back"] == 0


@pytest.mark.parametrize("kappa", [1e2, 1e4, 1e6, 1e8])
def test_conditioning_sweep_n8192_against_oracle(sl, orc, gpu_required, kappa):
    import torch

    n, nrhs = 8192, 4
    g = torch.Generator(device="cuda").manual_seed(2024 + 31 + int(np.log10(kappa)))
    s = torch.logspace(0.0, -float(np.log10(kappa)), n, dtype=torch.float64, device="cuda")
    A = torch.diag(s)
    for side in (0, 1):
        for _ in range(64):
            v = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 0.5
            tau = 2.0 / float(v @ v)
            if side == 0:
                A -= tau * torch.outer(v, v @ A)
            else:
                A -= tau * torch.outer(A @ v, v)
    At = A.T.contiguous()
    Bt = torch.rand((nrhs, n), dtype=torch.float64, device="cuda", generator=g) * 2.0 - 1.0
    Xt = torch.zeros_like(Bt)
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    info, it, st = sl.dgesv_ir_dev(n, nrhs, At.data_ptr(), n, piv.data_ptr(), Bt.data_ptr(), n,
                                   Xt.data_ptr(), n, fmt="bf16x3", nb=256, tol=1.0, keep_a=True)
    assert info == 0, st
    r = orc.sresid(_host(At), _host(Bt), _host(Xt))
    assert r < 16.0, (kappa, r, st)
    if kappa <= 1e6:
        assert st["fell_back"] == 0, (kappa, st)


@pytest.mark.parametrize("mode", [0, 1])
def test_batched_4096_systems_against_oracle(sl, orc, gpu_required, mode):
    import torch

    count = 4096
    rng = np.random.default_rng(2024 + 5)
    ns = rng.integers(16, 513, size=count)
    rs = rng.integers(1, 9, size=count)
    g = torch.Generator(device="cuda").manual_seed(2024 + 5)
    dA, dB, dX = [], [], []
    for i in range(count):
        n, r = int(ns[i]), int(rs[i])
        a = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=g) - 0.5
        if i % 2 == 0:
            a.diagonal().add_(n / 4.0)
        dA.append(a)
        dB.append(torch.rand((r, n), dtype=torch.float64, device="cuda", generator=g) - 0.5)
        dX.append(torch.zeros((r, n), dtype=torch.float64, device="cuda"))
    systems = [(dA[i].data_ptr(), int(ns[i]), int(ns[i]), dB[i].data_ptr(), int(ns[i]),
                int(rs[i]), dX[i].data_ptr(), int(ns[i])) for i in range(count)]
    plan = sl.BatchPlan(systems, mode=mode, tol=1.0, autotune=True)
    try:
        plan.execute()
        info, its, sr = plan.results()
    finally:
        plan.close()
    torch.cuda.synchronize()
    assert not np.any(np.array(info))
    worst = 0.0
    for i in range(count):
        r = orc.sresid(_host(dA[i]), _host(dB[i]), _host(dX[i]))
        worst = max(worst, r)
        assert r < 16.0, (i, int(ns[i]), int(rs[i]), r)
    assert worst < 16.0
