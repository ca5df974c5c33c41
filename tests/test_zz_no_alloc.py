"""The search entry point that allocates no device memory.

``lgb_match_search_static_scratch`` serves callers that cannot call cudaMalloc
(code inside a host application that owns all device memory through its own
pool, or that must avoid the implicit synchronisation of cudaMalloc/cudaFree).
Its scratch is a fixed 32 MiB array inside the library; the caller passes all
inputs and outputs.  This test calls it through the C ABI twice in a row and
checks both results against the allocating entry point (``lgb_match_search``
with a caller-provided workspace, via ``MatchTemplateSearch``), within the
tolerances of the other GPU tests, and checks that an over-size problem is
rejected before any GPU work.  It lives in its own file, collected last, and
passes alone in a fresh process as well as after the other tests.
"""

import ctypes

import pytest
import torch

from leopard_em_gb300 import _native
from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300.backend import MatchTemplateSearch

pytestmark = pytest.mark.gpu

MIP_RTOL = 1e-4
Z_ATOL = 1e-3


def _inputs():
    cfg = sy.MatchConfig(image_shape=(256, 256), template_size=32, n_blobs=60, blob_radius=11.0,
                         n_particles=2, snr=0.5, seed=21, defocus_offsets=(-150.0, 150.0))
    eul = sy.uniform_euler_grid(30.0, 30.0)[:10]
    return sy.make_match_workload(cfg, euler_angles=eul).kwargs


def _static_scratch_search(search: MatchTemplateSearch):
    """Run the whole search through lgb_match_search_static_scratch into fresh maps."""
    L = _native.lib()
    H, W = search.shape
    dev = search.device
    mip = torch.empty((H, W), dtype=torch.float32, device=dev)
    best = torch.empty((H, W), dtype=torch.int32, device=dev)
    s1 = torch.empty((H, W), dtype=torch.float64, device=dev)
    s2 = torch.empty((H, W), dtype=torch.float64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _native.check(L.lgb_match_init_stats(H * W, mip.data_ptr(), best.data_ptr(), s1.data_ptr(), s2.data_ptr(),
                                         stream), "init")
    _native.check(
        L.lgb_match_search_static_scratch(
            ctypes.byref(search.problem), search.image_dft.data_ptr(), search.template_dft.data_ptr(),
            search.projective_filters.data_ptr(), search.euler_angles.data_ptr(), 0,
            search.problem.n_orientations, mip.data_ptr(), best.data_ptr(), s1.data_ptr(), s2.data_ptr(), stream),
        "lgb_match_search_static_scratch",
    )
    torch.cuda.synchronize(dev)
    return mip, best, s1, s2


def test_static_scratch_search_matches_allocating_entry_point_twice():
    assert torch.cuda.is_available()
    kw = _inputs()
    ref = MatchTemplateSearch(**kw, device=torch.device("cuda:0"), orientation_batch_size=4)
    assert ref.workspace.numel() <= _native.lib().lgb_static_scratch_capacity()
    ref.run()
    torch.cuda.synchronize()
    n = ref.total_projections
    ref_mean = ref.corr_sum / n
    ref_std = torch.sqrt(torch.clamp(ref.corr_sq_sum / n - ref_mean**2, min=0))
    ref_z = (ref.mip.double() - ref_mean) / ref_std
    for _ in range(2):  # two calls in a row share (and reuse) the static scratch
        mip, best, s1, s2 = _static_scratch_search(ref)
        scale = ref.mip.double().abs().clamp_min(1.0)
        assert ((mip.double() - ref.mip.double()).abs() / scale).max().item() <= MIP_RTOL
        assert torch.equal(best, ref.best_index)
        mean = s1 / n
        std = torch.sqrt(torch.clamp(s2 / n - mean**2, min=0))
        z = (mip.double() - mean) / std
        assert (z - ref_z).abs().max().item() <= Z_ATOL
        assert ((mean - ref_mean).abs() / ref_std).max().item() <= 1e-4


def test_static_scratch_rejects_oversize_problem():
    L = _native.lib()
    big = _native.MatchProblem(4096, 4096, 384, 1, 3, 1000, 8)  # ~1.9 GB of scratch
    rc = L.lgb_match_search_static_scratch(ctypes.byref(big), None, None, None, None, 0, 1, None, None, None, None,
                                           None)
    assert rc == _native.LGB_ERR_WORKSPACE_TOO_SMALL
