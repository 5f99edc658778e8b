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
    dt = torch.bfloat16 if fmt == 0 else torch.float16
    mx = U.abs().amax(dim=0)
    e = torch.where(mx > 0, torch.frexp(mx)[1], torch.zeros_like(mx, dtype=torch.int32))
    Us = (U * torch.ldexp(torch.ones_like(mx), -e)).to(dt).double()
    L16 = L.to(dt).double()
    prod = (L16 @ Us) * torch.ldexp(torch.ones_like(mx, dtype=torch.float64), e.to(torch.float64).int())
    bound = (L16.abs() @ Us.abs()) * torch.ldexp(torch.ones_like(mx, dtype=torch.float64), e.int())
    return C.double() - prod, bound


@pytest.mark.parametrize("fmt", [0, 1])
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
