"""Precision form: the split-precision tcgen05 GEMM against FP64 products.

Tolerances (relative to max |D|): three-term BF16 split 2e-5, FP16 split 2e-6
(each hi/lo part keeps 8 / 11 significant bits, so the split operands carry
~16 / ~22 and the dropped lo*lo term sits below FP32 rounding); one-term BF16
5e-3 (8 bits).
"""

import pytest
import torch

from leopard_em_gb300 import precision as pr

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    yield


@pytest.mark.parametrize(
    "M,N,K,bn,f16,terms,tol",
    [
        (128, 256, 64, 256, False, 3, 2e-5),     # one tile, one K chunk
        (256, 300, 192, 256, False, 3, 2e-5),    # ragged N, three chunks (pipeline reload)
        (384, 200, 1024, 128, False, 3, 2e-5),   # 16 chunks, N tile 128
        (128, 512, 128, 256, True, 3, 2e-6),     # FP16 split
        (256, 256, 256, 256, False, 1, 5e-3),    # hi only
    ],
)
def test_tc_gemm_against_fp64(M, N, K, bn, f16, terms, tol):
    g = torch.Generator(device="cpu").manual_seed(M + N + K)
    a = torch.randn(M, K, generator=g, dtype=torch.float64)
    b = torch.randn(N, K, generator=g, dtype=torch.float64)
    ref = a @ b.T
    d = pr.tc_gemm(a.float().to(DEV), b.float().to(DEV), bn=bn, f16=f16, terms=terms).double().cpu()
    # the FP32 inputs themselves round at 2^-24; compare against their exact product
    ref32 = a.float().double() @ b.float().double().T
    err = (d - ref32).abs().max().item() / ref32.abs().max().item()
    assert err <= tol, f"relative error {err:.3e}"
    assert (d - ref).abs().max().item() / ref.abs().max().item() <= tol + 1e-6
