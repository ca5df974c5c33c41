"""Manager-level API: config pins from the reference's tests and an end-to-end
run of MatchTemplateManager / RefineTemplateManager (GPU)."""

import pytest
import torch

from leopard_em_gb300 import managers as m
from leopard_em_gb300 import synthetic as sy


def test_defocus_values_pin():
    """The reference pins -1000..1000 step 100 -> 21 values (test_defocus_search.py:25-63)."""
    cfg = m.DefocusSearchConfig(defocus_min=-1000.0, defocus_max=1000.0, defocus_step=100.0)
    assert torch.allclose(cfg.defocus_values, torch.arange(-1000, 1001, 100, dtype=torch.float32))
    assert m.DefocusSearchConfig(enabled=False).defocus_values.tolist() == [0.0]
    with pytest.raises(ValueError):
        m.DefocusSearchConfig(defocus_min=100.0, defocus_max=-100.0).defocus_values
    with pytest.raises(ValueError):
        m.DefocusSearchConfig(defocus_step=0.0)


def test_search_tensors_insert_zero():
    vals = m.get_search_tensors(-150.0, 150.0, 100.0)
    assert 0.0 in vals.tolist() and vals.tolist() == sorted(vals.tolist())
    assert 0.0 not in m.get_search_tensors(-150.0, 150.0, 100.0, skip_enforce_zero=True).tolist()


def test_valid_cropping_and_backend_kwargs_shapes():
    img = torch.randn(128, 128)
    vol, _ = sy.blob_volume(32, 40, 1.5, 10.0, 0)
    mgr = m.MatchTemplateManager(micrograph=img, template_volume=vol,
                                 orientation_search_config=m.OrientationSearchConfig(psi_step=60, theta_step=60),
                                 defocus_search_config=m.DefocusSearchConfig(defocus_min=-200, defocus_max=200,
                                                                             defocus_step=200))
    kw = mgr.make_backend_core_function_kwargs()
    assert kw["image_dft"].shape == (128, 65) and kw["template_dft"].shape == (32, 32, 17)
    assert kw["ctf_filters"].shape == (1, 3, 32, 17) and kw["whitening_filter_template"].shape == (32, 17)
    r = m.MatchTemplateResult(**{k: torch.zeros(128, 128) for k in
                                 ["mip", "scaled_mip", "correlation_average", "correlation_variance",
                                  "orientation_psi", "orientation_theta", "orientation_phi", "relative_defocus"]})
    r.apply_valid_cropping((32, 32))
    assert r.mip.shape == (97, 97) and r.relative_defocus.shape == (97, 97)


@pytest.mark.gpu
def test_match_manager_finds_planted_particle():
    cfg = sy.MatchConfig(image_shape=(256, 256), template_size=32, n_blobs=60, blob_radius=11.0, n_particles=1,
                         snr=1.0, seed=4, out_of_plane_step=30.0, in_plane_step=30.0)
    wl = sy.make_match_workload(cfg, keep_image=True)
    vol, _ = sy.blob_volume(32, 60, 1.5, 11.0, 4)
    mgr = m.MatchTemplateManager(
        micrograph=wl.image, template_volume=vol,
        optics_group=m.OpticsGroup(pixel_size=1.0, defocus_u=12000.0, defocus_v=12000.0),
        defocus_search_config=m.DefocusSearchConfig(enabled=False),
        orientation_search_config=m.OrientationSearchConfig(psi_step=30.0, theta_step=30.0))
    mgr.run_match_template(orientation_batch_size=8, do_result_export=False)
    r = mgr.match_template_result
    assert r.mip.shape == (225, 225)
    y0, x0, oi, eul = wl.planted[0]
    # ~130 orientations: per-pixel z is too noisy to rank; the MIP peak is the particle
    py, px = divmod(int(r.mip.argmax()), r.mip.shape[1])
    assert abs(py - y0) <= 1 and abs(px - x0) <= 1
    assert (float(r.orientation_phi[y0, x0]), float(r.orientation_theta[y0, x0]),
            float(r.orientation_psi[y0, x0])) == pytest.approx(eul)
    # peak picking on the device at a cutoff just under the particle's z
    peaks = r.locate_peaks(z_score_cutoff=float(r.scaled_mip[y0, x0]) - 1e-3, mask_radius=5.0)
    d2 = (peaks.pos_y - y0) ** 2 + (peaks.pos_x - x0) ** 2
    assert int(d2.min()) < 25  # the particle is picked or suppressed by a higher-z neighbour
    assert bool((peaks.scaled_mip[1:] <= peaks.scaled_mip[:-1]).all())  # descending z
    assert peaks.total_correlations == r.total_projections
    assert set(r.peaks_to_dict()) >= {"pos_y", "pos_x", "mip", "scaled_mip", "psi", "relative_defocus"}


@pytest.mark.gpu
def test_refine_manager_runs_and_keeps_keys():
    kw, truth = sy.make_refine_workload(sy.RefineConfig(crop=128, template_size=64, n_blobs=100, blob_radius=20.0,
                                                        snr_range=(0.5, 0.5)), 2)
    imgs = torch.fft.irfftn(kw["particle_stack_dft"], s=(128, 128), dim=(-2, -1))
    vol, _ = sy.blob_volume(64, 100, 1.2, 20.0, 0)
    mgr = m.RefineTemplateManager(
        particle_images=imgs, template_volume=vol, euler_angles=kw["euler_angles"], defocus_u=kw["defocus_u"],
        defocus_v=kw["defocus_v"], defocus_angle=kw["defocus_angle"],
        optics_group=m.OpticsGroup(pixel_size=1.06),
        orientation_refinement_config=m.RefineOrientationConfig(psi_step_coarse=2.0, psi_step_fine=1.0,
                                                                theta_step_coarse=2.0, theta_step_fine=1.0))
    res = mgr.run_refine_template(orientation_batch_size=16)
    assert set(res) >= {"refined_z_score", "refined_euler_angles", "refined_pos_y", "angle_idx"}
    assert res["refined_euler_angles"].shape == (2, 3)


@pytest.mark.gpu
def test_preprocessing_on_the_gpu_matches_the_host():
    """make_backend_core_function_kwargs on the GPU gives the host's inputs."""
    img = torch.randn(256, 288, generator=torch.Generator().manual_seed(2))
    vol, _ = sy.blob_volume(32, 40, 1.5, 10.0, 0)
    mgr = m.MatchTemplateManager(micrograph=img, template_volume=vol,
                                 orientation_search_config=m.OrientationSearchConfig(psi_step=60, theta_step=60),
                                 defocus_search_config=m.DefocusSearchConfig(defocus_min=-200, defocus_max=200,
                                                                             defocus_step=200))
    host = mgr.make_backend_core_function_kwargs()
    dev = mgr.make_backend_core_function_kwargs(preprocess_device="cuda:0")
    for k in ("image_dft", "template_dft", "ctf_filters", "whitening_filter_template"):
        assert dev[k].is_cuda, k
        a, b = host[k], dev[k].cpu()
        assert a.shape == b.shape, k
        assert (a - b).abs().max().item() <= 1e-4 * max(1.0, a.abs().max().item()), k
