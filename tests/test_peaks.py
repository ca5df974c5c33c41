"""Z-score peak picking: the oracle against vectors recorded from the
reference's own analysis/zscore_metric.py and analysis/utils.py (CPU), and the
device kernel (lgb_peaks_find) against the oracle (GPU).  Positions must match
exactly, in the same order."""

import os

import numpy as np
import pytest
import torch

from oracle import ref_peaks as orp

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "peaks_small.npz"))
CASES = [(m, c, r) for m in ("p1", "p2", "p3") for c, r in ((3.0, 5.0), (2.0, 2.5), (4.0, 10.0))]


@pytest.mark.parametrize("name,cutoff,radius", CASES)
def test_oracle_matches_reference_peaks(name, cutoff, radius):
    z = torch.from_numpy(GOLD[f"{name}/z"])
    py, px = orp.find_peaks_from_zscore(z, cutoff, radius)
    key = f"{name}/c{cutoff}/r{radius}"
    np.testing.assert_array_equal(py.numpy(), GOLD[f"{key}/pos_y"])
    np.testing.assert_array_equal(px.numpy(), GOLD[f"{key}/pos_x"])


def test_oracle_cutoff_matches_reference():
    vals = [orp.gaussian_noise_zscore_cutoff(int(n), fp) for n in GOLD["cutoff/num_ccg"] for fp in (1.0, 0.5)]
    np.testing.assert_allclose(vals, GOLD["cutoff/value"], rtol=1e-12)


def _tie_map(seed=4, H=70, W=90):
    g = torch.Generator().manual_seed(seed)
    z = torch.randn(H, W, generator=g) * 3
    return torch.round(z * 2) / 2  # many exact ties


@pytest.mark.gpu
@pytest.mark.parametrize("name,cutoff,radius", CASES)
def test_device_matches_golden(name, cutoff, radius):
    from leopard_em_gb300 import peaks

    z = torch.from_numpy(GOLD[f"{name}/z"])
    py, px = peaks.find_peaks_from_zscore(z, cutoff, radius, device="cuda:0")
    key = f"{name}/c{cutoff}/r{radius}"
    np.testing.assert_array_equal(py.numpy(), GOLD[f"{key}/pos_y"])
    np.testing.assert_array_equal(px.numpy(), GOLD[f"{key}/pos_x"])


@pytest.mark.gpu
@pytest.mark.parametrize("cutoff,radius", [(1.0, 5.0), (0.0, 3.0), (2.0, 7.5), (-1.0, 1.0)])
def test_device_matches_oracle_with_ties_and_edges(cutoff, radius):
    from leopard_em_gb300 import peaks

    z = _tie_map()
    py, px = peaks.find_peaks_from_zscore(z, cutoff, radius, device="cuda:0")
    ry, rx = orp.find_peaks_from_zscore(z, cutoff, radius)
    np.testing.assert_array_equal(py.numpy(), ry.numpy())
    np.testing.assert_array_equal(px.numpy(), rx.numpy())


@pytest.mark.gpu
def test_device_on_a_search_map_and_statistics():
    """Peaks of a 4096^2-sized map with planted bumps; extract_peaks_and_statistics_zscore gathers the maps."""
    from leopard_em_gb300 import peaks

    g = torch.Generator().manual_seed(9)
    H = W = 1024
    z = torch.randn(H, W, generator=g)
    ys = torch.randint(0, H, (300,), generator=g)
    xs = torch.randint(0, W, (300,), generator=g)
    z[ys, xs] += 9.0
    cut = peaks.gaussian_noise_zscore_cutoff(H * W * 1000)
    py, px = peaks.find_peaks_from_zscore(z, cut, 5.0, device="cuda:0")
    ry, rx = orp.find_peaks_from_zscore(z, cut, 5.0)
    np.testing.assert_array_equal(py.numpy(), ry.numpy())
    np.testing.assert_array_equal(px.numpy(), rx.numpy())
    maps = [torch.rand(H, W, generator=g) for _ in range(8)]
    res = peaks.extract_peaks_and_statistics_zscore(maps[0], z, *maps[1:7], total_correlation_positions=1000,
                                                    mask_radius=5.0, device="cuda:0")
    assert torch.equal(res.pos_y, py) and torch.equal(res.psi, maps[1][py, px])
    assert res.total_correlations == 1000


@pytest.mark.gpu
def test_device_no_candidates_and_errors():
    from leopard_em_gb300 import peaks

    z = torch.zeros(32, 32)
    py, px = peaks.find_peaks_from_zscore(z, 1.0, 5.0, device="cuda:0")
    assert py.numel() == 0 and px.numel() == 0
    with pytest.raises(ValueError):
        peaks.find_peaks_from_zscore(torch.zeros(4, 4, 4), 1.0, 5.0, device="cuda:0")
    with pytest.raises(ValueError):
        peaks.find_peaks_from_zscore(z, 1.0, -1.0, device="cuda:0")
