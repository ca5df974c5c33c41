"""Batched form: zero-padded grids for micrographs of any size, CUDA-graph
replay, the autotuner and the many-micrograph driver.

Acceptance as in test_match_gpu.py (MIP 1e-4 of max(|MIP|, 1); argmax equal
where the oracle's top two differ by more than that; z within 1e-3; mean/std
within 1e-3 of the std).  A micrograph whose size is not a compiled FFT length
is searched on the next compiled grid with zero padding; the reference's
circular correlation and the padded search agree at the valid positions
y <= H - d, x <= W - d, which is where parity is asserted for those.
"""

import numpy as np
import pytest
import torch

from leopard_em_gb300 import autotune
from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300.backend import MatchTemplateSearch
from leopard_em_gb300.backend.batched import match_template_batch
from leopard_em_gb300.backend.core_match_template import padded_grid
from oracle import ref_match_template as orc

pytestmark = pytest.mark.gpu

MIP_RTOL = 1e-4
Z_ATOL = 1e-3
DEV = torch.device("cuda:0")


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    yield


def _workload(H, W, d, n_o, n_df=1, n_cs=1, seed=5):
    cfg = sy.MatchConfig(image_shape=(H, W), template_size=d, n_blobs=60, blob_sigma=1.5, blob_radius=d * 0.35,
                         n_particles=3, snr=0.5, seed=seed,
                         defocus_offsets=tuple(np.linspace(-300, 300, n_df).tolist()) if n_df > 1 else (0.0,),
                         pixel_size_offsets=tuple(np.linspace(-0.02, 0.02, n_cs).tolist()) if n_cs > 1 else (0.0,))
    eul = sy.uniform_euler_grid(30.0, 30.0)
    idx = torch.randperm(eul.shape[0], generator=torch.Generator().manual_seed(seed))[:n_o]
    return sy.make_match_workload(cfg, euler_angles=eul[idx]).kwargs


def _search(kw, batch, **opts):
    s = MatchTemplateSearch(**kw, device=DEV, orientation_batch_size=batch, **opts)
    s.run()
    res = s.result(to_cpu=True)
    H, W = res["mip"].shape
    res["best_global_index"] = s.maps()["best_global_index"][:H, :W].cpu()
    res["_maps"] = {k: v.clone() for k, v in s.maps().items()}
    torch.cuda.synchronize()
    return res


def _assert_parity(gpu, ref, rows, cols):
    sl = (slice(0, rows), slice(0, cols))
    mip_r = ref["mip"][sl].double()
    scale = mip_r.abs().clamp_min(1.0)
    rel = ((gpu["mip"][sl].double() - mip_r).abs() / scale).max().item()
    assert rel <= MIP_RTOL, f"MIP relative error {rel:.3e}"
    sep = (mip_r - ref["second_best"][sl].double()) > MIP_RTOL * scale
    bad = (gpu["best_global_index"][sl].long() != ref["best_global_index"][sl].long()) & sep
    assert sep.float().mean() > 0.5
    assert int(bad.sum()) == 0, f"{int(bad.sum())} separated pixels with a different argmax"
    dz = (gpu["scaled_mip"][sl].double() - ref["scaled_mip"][sl].double()).abs().max().item()
    assert dz <= Z_ATOL, f"z-score error {dz:.3e}"
    std = ref["correlation_variance"][sl].double()
    dm = (gpu["correlation_mean"][sl].double() - ref["correlation_mean"][sl].double()).abs() / std.clamp_min(1e-6)
    ds = (gpu["correlation_variance"][sl].double() - std).abs() / std.clamp_min(1e-6)
    assert dm.max().item() <= 1e-3 and ds.max().item() <= 1e-3


def _oracle(kw, batch):
    return orc.core_match_template_cpu(**kw, orientation_batch_size=batch, backend="batched",
                                       stat_dtype=torch.float64, track_second_best=True)


@pytest.mark.parametrize(
    "H,W,d,n_o,n_df,batch",
    [
        # >= 16 samples per pixel: with millions of pixels, an 8-sample std is
        # small enough somewhere to amplify FP32 correlogram noise past 1e-3 in z
        (2880, 3072, 32, 16, 1, 8),  # new column length 2880, row length 3072 (1536-point half transform)
        (3840, 5760, 32, 16, 1, 8),  # column 3840 (16*16*5*3), row 5760 (2880-point half transform)
        (5760, 2880, 32, 16, 1, 8),  # column 5760: two columns per CTA (720 threads)
        (3072, 3840, 64, 8, 2, 4),   # column 3072, row 3840, two defocus planes (16 samples)
    ],
)
def test_compiled_micrograph_lengths_match_oracle(H, W, d, n_o, n_df, batch):
    kw = _workload(H, W, d, n_o, n_df)
    assert padded_grid(H, W) == (H, W)
    gpu = _search(kw, batch)
    ref = _oracle(kw, batch)
    _assert_parity(gpu, ref, H, W)


@pytest.mark.parametrize(
    "H,W,d,n_o,batch",
    [
        (250, 270, 32, 8, 4),      # -> 256 x 288
        (200, 130, 48, 8, 8),      # -> 256 x 256 (130 pads past 128)
        (3838, 3710, 64, 16, 8),   # a batched-form micrograph: -> 3840 x 3840
    ],
)
def test_padded_grid_matches_oracle_on_valid_region(H, W, d, n_o, batch):
    kw = _workload(H, W, d, n_o)
    Hp, Wp = padded_grid(H, W)
    assert (Hp, Wp) != (H, W) and Hp >= H and Wp >= W
    gpu = _search(kw, batch)
    assert tuple(gpu["mip"].shape) == (H, W)
    ref = _oracle(kw, batch)
    _assert_parity(gpu, ref, H - d + 1, W - d + 1)


def test_larger_grid_keeps_valid_region():
    """A compiled size searched on a larger (power-of-two) grid, as the tuner may choose."""
    H, W, d = 288, 288, 48
    kw = _workload(H, W, d, 16)
    gpu = _search(kw, 8, grid=(512, 512))
    assert tuple(gpu["_maps"]["mip"].shape) == (512, 512)
    ref = _oracle(kw, 8)
    _assert_parity(gpu, ref, H - d + 1, W - d + 1)
    with pytest.raises(ValueError):
        MatchTemplateSearch(**kw, device=DEV, grid=(256, 512))


@pytest.mark.parametrize("H,W,n_o,batch,graph_batches", [(256, 256, 41, 4, 3), (512, 512, 64, 8, 2),
                                                          (250, 270, 20, 3, 1)])
def test_graph_replay_is_bitwise_equal(H, W, n_o, batch, graph_batches):
    kw = _workload(H, W, 32, n_o, n_df=2)
    plain = _search(kw, batch)
    graph = _search(kw, batch, graph_batches=graph_batches)
    for k, v in plain["_maps"].items():
        assert torch.equal(v, graph["_maps"][k]), k


def test_col_waves_do_not_change_results():
    kw = _workload(512, 512, 48, 12)
    a = _search(kw, 4, col_waves=1)
    b = _search(kw, 4, col_waves=8)
    for k, v in a["_maps"].items():
        assert torch.equal(v, b["_maps"][k]), k


def test_autotuner_picks_valid_parameters_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv(autotune.CACHE_ENV, str(tmp_path / "tune.json"))
    kw = _workload(512, 512, 64, 24, n_df=2)
    t1 = autotune.tune_search(**kw, device=DEV, batches=(2, 4, 8), waves=(2, 4), n_probe=16)
    assert t1.orientation_batch in (2, 4, 8) and t1.col_waves in (2, 4) and t1.graph_batches >= 1
    assert t1.grid == (512, 512)  # the only candidate grid of a 512^2 micrograph
    assert t1.ms_per_orientation > 0
    assert (tmp_path / "tune.json").exists()
    t2 = autotune.tune_search(**kw, device=DEV, batches=(2, 4, 8), waves=(2, 4), n_probe=16)
    assert t2 == t1  # served from the cache
    # the tuned search gives the same MIP and indices as a plain batch-1 search
    tuned = _search(kw, t1.orientation_batch, col_waves=t1.col_waves, graph_batches=t1.graph_batches, grid=t1.grid)
    plain = _search(kw, 1)
    assert torch.equal(tuned["_maps"]["mip"], plain["_maps"]["mip"])
    assert torch.equal(tuned["_maps"]["best_global_index"], plain["_maps"]["best_global_index"])
    torch.testing.assert_close(tuned["_maps"]["correlation_sum"], plain["_maps"]["correlation_sum"], rtol=1e-5,
                               atol=1e-4)


def test_batched_driver_over_uneven_micrographs(tmp_path, monkeypatch):
    monkeypatch.setenv(autotune.CACHE_ENV, str(tmp_path / "tune.json"))
    base = sy.MatchConfig(template_size=32, n_blobs=60, blob_sigma=1.5, blob_radius=11.0, n_particles=3, snr=0.5,
                          defocus_offsets=(-200.0, 0.0, 200.0), pixel_size_offsets=(-0.02, 0.0, 0.02))
    template = sy.make_template(base)
    eul = sy.uniform_euler_grid(30.0, 30.0)[:20]
    mics = []
    for i, shape in enumerate([(256, 256), (250, 270), (288, 256), (256, 256)]):
        cfg = sy.MatchConfig(**{**base.__dict__, "image_shape": shape, "seed": 10 + i})
        kw = sy.make_match_workload(cfg, euler_angles=eul, template=template).kwargs
        mics.append({k: kw[k] for k in ("image_dft", "ctf_filters", "whitening_filter_template", "defocus_values",
                                        "pixel_values")})
    results, report = match_template_batch(mics, template[0], eul, DEV, orientation_range=(0, 16))
    assert len(results) == 4 and len(report.ms) == 4 and all(ms > 0 for ms in report.ms)
    assert report.percentile(50) <= report.percentile(99)
    for m, res, grid, tun in zip(mics, results, report.grids, report.tunings):
        # same grid and orientation as the driver chose (the tuner may pad past
        # the smallest grid, or search the transposed micrograph)
        single = MatchTemplateSearch(**m, template_dft=template[0], euler_angles=eul, device=DEV,
                                     orientation_batch_size=tun.orientation_batch, grid=grid,
                                     transpose=tun.transpose)
        single.run(0, 16)
        ref = single.result(to_cpu=True)
        H, wc = m["image_dft"].shape
        assert tuple(res["mip"].shape) == (H, 2 * (wc - 1))
        assert torch.equal(res["mip"], ref["mip"])
        torch.testing.assert_close(res["scaled_mip"], ref["scaled_mip"], rtol=1e-4, atol=1e-4)


@pytest.mark.parametrize("H,W,d,grid", [(256, 512, 48, None), (288, 250, 32, None), (288, 250, 32, (256, 512))])
def test_transposed_search_matches_oracle(H, W, d, grid):
    """A search of the transposed micrograph with the x/y-exchanged template and
    conjugated rotations equals the direct search (oracle) at valid positions:
    astigmatic CTF filters, orientations at theta = 0 and 180 included,
    compiled and zero-padded transposed grids."""
    from leopard_em_gb300 import preprocess as pp

    kw = _workload(H, W, d, 10, n_df=2, seed=9)
    kw["euler_angles"][0] = torch.tensor([30.0, 0.0, 40.0])
    kw["euler_angles"][1] = torch.tensor([10.0, 180.0, 70.0])
    kw["ctf_filters"] = pp.ctf_filter_stack(d, 11000.0, 9000.0, kw["defocus_values"], kw["pixel_values"],
                                            astigmatism_angle=30.0)
    ref = _oracle(kw, 4)
    gpu = _search(kw, 4, transpose=True, grid=grid)
    assert gpu["mip"].shape == (H, W)
    _assert_parity(gpu, ref, H - d + 1, W - d + 1)
    for key in ("best_phi", "best_theta", "best_psi", "best_defocus"):
        sep = ref["mip"][: H - d + 1, : W - d + 1] - ref["second_best"][: H - d + 1, : W - d + 1] > 1e-3
        got = gpu[key][: H - d + 1, : W - d + 1]
        want = ref[key][: H - d + 1, : W - d + 1].to(got.dtype)
        assert bool((got[sep] == want[sep]).all()), key


def test_autotuner_may_pick_a_transposed_grid_and_keeps_results():
    """The tuner times both orientations of a non-square micrograph; whichever
    it picks, the batched driver's maps agree with the oracle."""
    kw = _workload(288, 128, 32, 8, seed=11)
    t = autotune.tune_search(kw["image_dft"], kw["template_dft"], kw["ctf_filters"], kw["whitening_filter_template"],
                             kw["defocus_values"], kw["pixel_values"], kw["euler_angles"], DEV, n_probe=8,
                             use_cache=False)
    assert isinstance(t.transpose, bool)
    mic = {k: kw[k] for k in ("image_dft", "ctf_filters", "whitening_filter_template", "defocus_values",
                               "pixel_values")}
    res, rep = match_template_batch([mic], kw["template_dft"], kw["euler_angles"], DEV, tune=True, tune_cache=False)
    ref = _oracle(kw, 4)
    r = res[0]
    sl = (slice(0, 288 - 32 + 1), slice(0, 128 - 32 + 1))
    scale = ref["mip"][sl].double().abs().clamp_min(1.0)
    assert ((r["mip"][sl].double() - ref["mip"][sl].double()).abs() / scale).max().item() <= MIP_RTOL
    assert (r["scaled_mip"][sl].double() - ref["scaled_mip"][sl].double()).abs().max().item() <= Z_ATOL
