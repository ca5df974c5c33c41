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


# ---------------------------------------------------------------------------
# The precision search against the FP64 oracle
# ---------------------------------------------------------------------------
import numpy as np  # noqa: E402

from leopard_em_gb300 import synthetic as sy  # noqa: E402
from leopard_em_gb300.backend import MatchTemplateSearch  # noqa: E402
from oracle import ref_match_template as orc  # noqa: E402


def _workload(H, W, d, n_o, n_df=1, seed=7):
    cfg = sy.MatchConfig(image_shape=(H, W), template_size=d, n_blobs=60, blob_sigma=1.5, blob_radius=d * 0.35,
                         n_particles=3, snr=0.5, seed=seed,
                         defocus_offsets=tuple(np.linspace(-300, 300, n_df).tolist()) if n_df > 1 else (0.0,))
    eul = sy.uniform_euler_grid(30.0, 30.0)
    idx = torch.randperm(eul.shape[0], generator=torch.Generator().manual_seed(seed))[:n_o]
    return sy.make_match_workload(cfg, euler_angles=eul[idx]).kwargs


def _run(kw, batch, precision):
    s = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=batch, precision=precision)
    s.run()
    res = s.result(to_cpu=True)
    res["best_global_index"] = s.best_index.cpu()
    return res


# Precision acceptance (the precision form's targets): MIP relative error <= 1e-3,
# z-score error <= 0.05, argmax equal where the FP64 oracle's top two differ by
# more than 1e-3 of the MIP scale.  The split operands do far better; the test
# also holds BF16x3 to 1e-4 / 5e-3 so a regression shows.
@pytest.mark.parametrize(
    "H,W,d,n_o,n_df,batch,precision,mip_tol,z_tol",
    [
        (512, 512, 64, 32, 1, 32, "bf16x3", 1e-4, 5e-3),   # the small configuration's image and template
        (256, 256, 32, 19, 2, 4, "bf16x3", 1e-4, 5e-3),    # two defocus planes, partial last batch
        (128, 256, 32, 16, 1, 8, "bf16x3", 1e-4, 5e-3),    # non-square
        (512, 512, 64, 32, 1, 32, "fp16x3", 1e-3, 0.05),
    ],
)
def test_precision_search_against_fp64_oracle(H, W, d, n_o, n_df, batch, precision, mip_tol, z_tol):
    kw = _workload(H, W, d, n_o, n_df)
    ref = orc.core_match_template_cpu(**{k: (v.double() if k in ("ctf_filters", "whitening_filter_template") else v)
                                         for k, v in kw.items()},
                                      orientation_batch_size=batch, backend="batched", stat_dtype=torch.float64,
                                      track_second_best=True, compute_dtype=torch.float64)
    got = _run(kw, batch, precision)
    mip_r = ref["mip"].double()
    scale = mip_r.abs().clamp_min(1.0)
    rel = ((got["mip"].double() - mip_r).abs() / scale).max().item()
    assert rel <= mip_tol, f"MIP relative error {rel:.3e}"
    sep = (mip_r - ref["second_best"].double()) > 1e-3 * scale
    bad = (got["best_global_index"].long() != ref["best_global_index"].long()) & sep
    assert sep.float().mean() > 0.5 and int(bad.sum()) == 0, f"{int(bad.sum())} separated pixels differ"
    dz = (got["scaled_mip"].double() - ref["scaled_mip"].double()).abs().max().item()
    assert dz <= z_tol, f"z error {dz:.3e}"


def test_precision_matches_plain_fp32_search():
    kw = _workload(256, 256, 32, 24, 1)
    plain = _run(kw, 8, "fp32")
    prec = _run(kw, 8, "bf16x3")
    scale = plain["mip"].double().abs().clamp_min(1.0)
    assert ((prec["mip"].double() - plain["mip"].double()).abs() / scale).max().item() <= 1e-4


def test_precision_rejects_unsupported_shapes():
    kw = _workload(4096, 4096, 64, 2)
    with pytest.raises(ValueError):
        MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=2, precision="bf16x3")
    kw = _workload(256, 256, 32, 40)
    with pytest.raises(ValueError):
        MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=40, precision="bf16x3")  # > 32 per batch
    with pytest.raises(ValueError):
        MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=8, precision="tf32")
