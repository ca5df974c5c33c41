"""Plan form of the C ABI (lgb_match_plan_*): create / set_filters / set_image
/ search in ranges / finalize / destroy gives the same maps as the stateless
calls behind MatchTemplateSearch (bit for bit), and bad shapes fail at create."""

import ctypes

import pytest
import torch

from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300._native import MatchProblem, check, lib
from leopard_em_gb300.backend import MatchTemplateSearch

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _kw():
    cfg = sy.MatchConfig(image_shape=(256, 288), template_size=32, n_blobs=60, blob_radius=11.0, n_particles=2,
                         snr=0.5, seed=6, defocus_offsets=(-200.0, 0.0, 200.0))
    eul = sy.uniform_euler_grid(30.0, 30.0)[:21]
    return sy.make_match_workload(cfg, euler_angles=eul).kwargs


def test_plan_equals_stateless_search():
    kw = _kw()
    ref = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=4)
    ref.run(0, 8)
    ref.run(8, 21)
    out_ref = ref.result(to_cpu=True)
    L = lib()
    H, W = 256, 288
    prob = MatchProblem(H, W, 32, 1, 3, 21, 4)
    st = ctypes.c_int(-1)
    plan = L.lgb_match_plan_create(ctypes.byref(prob), ctypes.byref(st))
    assert st.value == 0 and plan
    try:
        s = ctypes.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)
        d = {k: v.to(DEV).contiguous() for k, v in kw.items()}
        d["image_dft"] = d["image_dft"].to(torch.complex64)
        check(L.lgb_match_plan_set_filters(plan, d["ctf_filters"].data_ptr(),
                                           d["whitening_filter_template"].data_ptr(), s), "set_filters")
        check(L.lgb_match_plan_set_image(plan, d["image_dft"].data_ptr(), s), "set_image")
        for a, b in ((0, 8), (8, 21)):
            check(L.lgb_match_plan_search(plan, d["template_dft"].to(torch.complex64).data_ptr(),
                                          d["euler_angles"].float().data_ptr(), a, b, s), "search")
        outs = {k: torch.empty((H, W), device=DEV) for k in
                ("scaled_mip", "best_phi", "best_theta", "best_psi", "best_defocus", "correlation_mean",
                 "correlation_variance")}
        check(L.lgb_match_plan_finalize(plan, d["euler_angles"].float().data_ptr(),
                                        d["defocus_values"].float().data_ptr(),
                                        *[outs[k].data_ptr() for k in ("scaled_mip", "best_phi", "best_theta",
                                                                       "best_psi", "best_defocus",
                                                                       "correlation_mean",
                                                                       "correlation_variance")], s), "finalize")
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        check(L.lgb_match_plan_maps(plan, *[ctypes.byref(p) for p in ptrs]), "maps")
        assert all(p.value for p in ptrs)
        torch.cuda.synchronize()
        for k in outs:
            assert torch.equal(outs[k].cpu(), out_ref[k]), k
    finally:
        L.lgb_match_plan_destroy(plan)


def test_plan_create_rejects_bad_problems():
    L = lib()
    st = ctypes.c_int(0)
    bad = MatchProblem(6000, 4096, 64, 1, 1, 4, 2)  # no compiled 6000-row grid
    assert not L.lgb_match_plan_create(ctypes.byref(bad), ctypes.byref(st))
    assert st.value == 2
    bad = MatchProblem(256, 256, 0, 1, 1, 4, 2)
    assert not L.lgb_match_plan_create(ctypes.byref(bad), ctypes.byref(st))
    assert st.value == 1
    L.lgb_match_plan_destroy(None)  # no-op
