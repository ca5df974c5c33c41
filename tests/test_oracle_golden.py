"""The CPU oracle against golden vectors produced by the reference's own backend code.

The vectors come from ``tests/golden/make_golden.py`` (which imports the
reference's ``backend/cross_correlation.py``, ``backend/utils.py`` and
``backend/process_results.py``).  Passing here pins the oracle's restatement of
the Leopard-EM operation sequence; the GPU path is then checked against the
oracle in ``tests/test_match_gpu.py``.
"""

import os

import numpy as np
import pytest
import torch

from oracle import ref_match_template as orc

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "match_small.npz"))


def _inputs(case):
    keys = ["image_dft", "template_dft", "ctf_filters", "whitening_filter_template",
            "defocus_values", "pixel_values", "euler_angles"]
    return {k: torch.from_numpy(GOLD[f"{case}/in/{k}"]) for k in keys}


@pytest.mark.parametrize("case", ["a", "b"])
def test_first_batch_correlogram_matches_reference(case):
    inp = _inputs(case)
    b = int(GOLD[f"{case}/batch"])
    rot = orc.euler_to_rotmat_zyz(inp["euler_angles"][:b])
    pf = inp["ctf_filters"] * inp["whitening_filter_template"][None, None]
    ref = GOLD[f"{case}/cc_first_batch"]
    got_b = orc.cross_correlate_batched_cpu(inp["image_dft"], inp["template_dft"], rot, pf).numpy()
    got_s = orc.cross_correlate_streamed(inp["image_dft"], inp["template_dft"], rot, pf).numpy()
    scale = np.abs(ref).max()
    assert np.abs(got_b - ref).max() <= 1e-5 * scale
    assert np.abs(got_s - ref).max() <= 1e-4 * scale


@pytest.mark.parametrize("case", ["a", "b"])
@pytest.mark.parametrize("backend", ["batched", "streamed"])
def test_search_matches_reference(case, backend):
    inp = _inputs(case)
    b = int(GOLD[f"{case}/batch"])
    res = orc.core_match_template_cpu(**inp, orientation_batch_size=b, backend=backend)
    for key in ["mip", "scaled_mip", "correlation_mean", "correlation_variance"]:
        ref = GOLD[f"{case}/out/{key}"]
        np.testing.assert_allclose(res[key].numpy(), ref, rtol=2e-4, atol=2e-4 * np.abs(ref).max())
    agree = (res["best_global_index"].numpy() == GOLD[f"{case}/out/best_global_index"]).mean()
    assert agree > 0.995
    for key in ["best_phi", "best_theta", "best_psi", "best_defocus"]:
        assert (res[key].numpy() == GOLD[f"{case}/out/{key}"]).mean() > 0.995


def test_normalisation_matches_reference():
    p = torch.from_numpy(GOLD["norm/in"])
    got = orc.normalize_template_projection(p, (20, 20), (64, 96)).numpy()
    np.testing.assert_allclose(got, GOLD["norm/out"], rtol=1e-6, atol=1e-6)


def test_decode_matches_reference():
    gi = torch.from_numpy(GOLD["decode/gi"])
    eul = torch.from_numpy(GOLD["decode/euler"])
    dfv = torch.from_numpy(GOLD["decode/defocus"])
    got = torch.stack(orc.decode_global_search_index(gi, torch.zeros(2), dfv, eul)).numpy()
    np.testing.assert_array_equal(got, GOLD["decode/out"])


def test_projection_slice_theorem_fixes_rotation_convention():
    """Blob centres c project to (R^T c)_xy; R c would be far off."""
    d, sigma = 32, 2.5
    rng = np.random.default_rng(1)
    cent = rng.uniform(-6, 6, size=(8, 3))
    g = np.arange(d) - d // 2
    vol = np.zeros((d, d, d))
    for cx, cy, cz in cent:
        vol += np.exp(-((g[:, None, None] - cz) ** 2 + (g[None, :, None] - cy) ** 2
                        + (g[None, None, :] - cx) ** 2) / (2 * sigma**2))
    vdft = orc.volume_to_rfft_fourier_slice(torch.tensor(vol))
    R = orc.euler_to_rotmat_zyz(torch.tensor([[30.0, 40.0, 50.0]]), dtype=torch.float64)
    fs = torch.fft.ifftshift(orc.extract_central_slices_rfft_3d(vdft, R), dim=(-2,))
    proj = torch.fft.ifftshift(torch.fft.irfft2(fs), dim=(-2, -1))[0].numpy()
    good = orc.analytic_blob_projection(cent, sigma, R[0].numpy(), d)
    bad = orc.analytic_blob_projection(cent, sigma, R[0].numpy().T, d)
    err_good = np.abs(proj - good).max() / np.abs(good).max()
    err_bad = np.abs(proj - bad).max() / np.abs(bad).max()
    assert err_good < 0.2 and err_bad > 3 * err_good


# ---------------------------------------------------------------------------
# refinement (core_refine_template.py:555-767) against the reference's own code
# ---------------------------------------------------------------------------
from oracle import ref_refine_template as orr  # noqa: E402

RGOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "refine_small.npz"))


def refine_golden_inputs():
    keys = ["particle_stack_dft", "template_dft", "euler_angles", "euler_angle_offsets", "defocus_offsets",
            "pixel_size_offsets", "defocus_u", "defocus_v", "defocus_angle", "corr_mean", "corr_std",
            "projective_filters"]
    kw = {k: torch.from_numpy(RGOLD[f"in/{k}"]) for k in keys}
    ctf = {k.split("/", 1)[1]: RGOLD[k].item() for k in RGOLD.files if k.startswith("ctf/")}
    ctf.update(template_shape=(kw["template_dft"].shape[1], kw["template_dft"].shape[1]), even_zernikes=None,
               odd_zernikes=None, mag_matrix=None)
    kw["ctf_kwargs"] = ctf
    return kw, int(RGOLD["in/batch_size"])


def test_refine_single_particle_matches_reference():
    kw, b = refine_golden_inputs()
    for i in range(kw["particle_stack_dft"].shape[0]):
        st = orr.refine_single_particle(
            kw["particle_stack_dft"][i], kw["template_dft"], kw["euler_angles"][i], kw["euler_angle_offsets"],
            kw["defocus_u"][i], kw["defocus_v"][i], kw["defocus_angle"][i], kw["defocus_offsets"],
            kw["pixel_size_offsets"], kw["corr_mean"][i], kw["corr_std"][i], kw["ctf_kwargs"],
            kw["projective_filters"][i], b)
        for k in ["max_cc", "max_z_score"]:
            assert abs(st[k] - RGOLD[f"out/{k}"][i]) <= 1e-4 * abs(RGOLD[f"out/{k}"][i])
        for k in ["refined_phi_offset", "refined_theta_offset", "refined_psi_offset", "refined_defocus_offset",
                  "refined_pixel_size_offset", "refined_pos_y", "refined_pos_x", "angle_idx"]:
            assert st[k] == RGOLD[f"out/{k}"][i], k


def test_rotmat_euler_round_trip():
    e = torch.tensor([[10.0, 40.0, 300.0], [200.0, 120.0, 15.0], [359.0, 179.0, 1.0]], dtype=torch.float64)
    back = orr.rotmat_to_euler_zyz(orc.euler_to_rotmat_zyz(e, dtype=torch.float64))
    back = torch.where(back < 0, back + 360, back)
    assert torch.allclose(back, e, atol=1e-9)
