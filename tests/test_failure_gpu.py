"""Failure handling without GPU faults: the bounded device wait's expiry path,
host-side errors between orientation batches, and checkpoint / resume of a
search at a batch boundary."""

import ctypes
import time

import pytest
import torch

from leopard_em_gb300 import precision as pr
from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300._native import check, lib
from leopard_em_gb300.backend import MatchTemplateSearch

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _kw(n_o=24):
    cfg = sy.MatchConfig(image_shape=(256, 256), template_size=32, n_blobs=60, blob_radius=11.0, n_particles=2,
                         snr=0.5, seed=9, defocus_offsets=(-200.0, 0.0, 200.0))
    return sy.make_match_workload(cfg, euler_angles=sy.uniform_euler_grid(30.0, 30.0)[:n_o]).kwargs


def test_bounded_wait_expires_and_reports():
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    s = ctypes.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)
    t0 = time.perf_counter()
    check(lib().lgb_wait_timeout_selftest(4096, status.data_ptr(), s), "lgb_wait_timeout_selftest")
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 10.0
    assert int(status.item()) == 5  # LGB_ERR_DEVICE_TIMEOUT
    # the context is still usable: a tensor-core GEMM right after
    a = torch.randn(128, 64, device=DEV)
    b = torch.randn(256, 64, device=DEV)
    d = pr.tc_gemm(a, b).double().cpu()
    ref = a.double().cpu() @ b.double().cpu().T
    assert (d - ref).abs().max().item() <= 2e-5 * ref.abs().max().item()
    with pytest.raises(ValueError):
        check(lib().lgb_wait_timeout_selftest(0, status.data_ptr(), s), "bad poll count")


def test_error_between_batches_leaves_search_usable():
    kw = _kw()
    clean = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=4)
    clean.run(0, 16)
    s = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=4)
    s.run(0, 8)
    with pytest.raises(ValueError):
        s.run(8, 1000)  # outside the orientation set: rejected before any launch
    s.run(8, 16)
    for k, v in clean.maps().items():
        assert torch.equal(v, s.maps()[k]), k


def test_checkpoint_resume_at_batch_boundary(tmp_path):
    kw = _kw()
    full = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=4, graph_batches=2)
    full.run()
    ref = full.result(to_cpu=True)
    first = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=4)
    first.run(0, 12)
    torch.save(first.state_dict(), tmp_path / "state.pt")
    del first
    second = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=4)
    second.load_state_dict(torch.load(tmp_path / "state.pt"))
    second.run(12, 24)
    got = second.result(to_cpu=True)
    for k in ("mip", "scaled_mip", "best_phi", "best_psi", "best_defocus", "correlation_mean",
              "correlation_variance"):
        assert torch.equal(got[k], ref[k]), k
    other = MatchTemplateSearch(**_kw(20), device=DEV, orientation_batch_size=4)
    with pytest.raises(ValueError):
        other.load_state_dict(torch.load(tmp_path / "state.pt"))
