"""Manager-level API: the configuration pins of the reference's tests, YAML
round trips of the reference's configuration schema, and end-to-end runs of
MatchTemplateManager / RefineTemplateManager driven by YAML files (GPU)."""

import os

import numpy as np
import pytest
import torch

from leopard_em_gb300 import config_models as cm
from leopard_em_gb300 import managers as m
from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300.mrc import write_mrc
from leopard_em_gb300.particle_stack import MATCH_TEMPLATE_DF_COLUMN_ORDER, write_particle_table

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
REF_PROGRAMS = "/root/reference/programs"


# ---------------------------------------------------------------------------
# configuration pins (tests/pydantic_models/test_*.py of the reference)
# ---------------------------------------------------------------------------


def test_defocus_values_pin():
    """-1000..1000 step 100 -> 21 values (test_defocus_search.py:25-63)."""
    cfg = m.DefocusSearchConfig(defocus_min=-1000.0, defocus_max=1000.0, defocus_step=100.0)
    assert torch.allclose(cfg.defocus_values, torch.arange(-1000, 1001, 100, dtype=torch.float32))
    assert m.DefocusSearchConfig(enabled=False).defocus_values.tolist() == [0.0]
    with pytest.raises(ValueError):
        m.DefocusSearchConfig(defocus_min=100.0, defocus_max=-100.0).defocus_values
    with pytest.raises(cm.ValidationError, match="greater than 0"):
        m.DefocusSearchConfig(defocus_step=0.0)


def test_search_tensors_insert_zero():
    vals = m.get_search_tensors(-150.0, 150.0, 100.0)
    assert 0.0 in vals.tolist() and vals.tolist() == sorted(vals.tolist())
    assert 0.0 not in m.get_search_tensors(-150.0, 150.0, 100.0, skip_enforce_zero=True).tolist()


def test_orientation_grid_pins():
    """(24, 3) for psi/theta steps of 90 (test_orientation_search.py:99-110) and
    (42, 3) for the local grid psi 1.5/0.5, theta 2.5/1.0
    (test_orientation_search.py:179-196)."""
    assert m.OrientationSearchConfig(psi_step=90.0, theta_step=90.0).euler_angles.shape == (24, 3)
    cfg = m.RefineOrientationConfig(psi_step_coarse=1.5, psi_step_fine=0.5, theta_step_coarse=2.5,
                                    theta_step_fine=1.0, base_grid_method="uniform")
    off = cfg.euler_angles_offsets
    assert isinstance(off, torch.Tensor) and off.shape == (42, 3)
    # every offset inside the coarse window, psi on its fine steps
    assert float(off[:, 1].abs().max()) <= 2.5 + 1e-6 and float(off[:, 2].abs().max()) <= 1.5 + 1e-6
    assert torch.allclose(torch.unique(off[:, 2]), torch.arange(-1.5, 1.51, 0.5))
    assert m.RefineOrientationConfig(enabled=False).euler_angles_offsets.shape == (1, 3)
    basic = m.RefineOrientationConfig(psi_step_coarse=1.0, psi_step_fine=0.5, theta_step_coarse=1.0,
                                      theta_step_fine=1.0, phi_step_coarse=1.0, phi_step_fine=1.0,
                                      base_grid_method="basic").euler_angles_offsets
    assert basic.shape == (3 * 3 * 5, 3)


def test_refine_orientation_defaults_and_ranges():
    """test_orientation_search.py:113-176: defaults and ge=0 validation."""
    c = m.RefineOrientationConfig()
    assert (c.psi_step_coarse, c.psi_step_fine, c.theta_step_coarse, c.theta_step_fine) == (1.5, 0.1, 2.5, 0.25)
    for name in ("psi_step_coarse", "psi_step_fine", "theta_step_coarse", "theta_step_fine"):
        with pytest.raises(cm.ValidationError, match="Input should be greater than or equal to 0"):
            m.RefineOrientationConfig(**{name: -1.0})
    with pytest.raises(cm.ValidationError, match="Input should be greater than or equal to 0"):
        m.OrientationSearchConfig(theta_step=-1.0)


def test_orientation_symmetry_and_ranges():
    """Symmetry and explicit ranges are exclusive (orientation_search.py:84-124)."""
    with pytest.raises(cm.ValidationError):
        m.OrientationSearchConfig(phi_min=0.0)
    with pytest.raises(cm.ValidationError):
        m.OrientationSearchConfig(symmetry=None)
    full = dict(symmetry=None, phi_min=0.0, phi_max=360.0, theta_min=0.0, theta_max=180.0, psi_min=0.0,
                psi_max=360.0, psi_step=90.0, theta_step=90.0)
    assert m.OrientationSearchConfig(**full).euler_angles.shape == (24, 3)
    c2 = m.OrientationSearchConfig(symmetry="C2", psi_step=90.0, theta_step=90.0).euler_angles
    assert c2.shape == (12, 3) and float(c2[:, 2].max()) < 180.0
    both = m.MultipleOrientationConfig(orientation_configs=[{"psi_step": 90.0, "theta_step": 90.0},
                                                            {"symmetry": "C2", "psi_step": 90.0,
                                                             "theta_step": 90.0}])
    assert both.euler_angles.shape == (36, 3)


def test_optics_and_computational_validation():
    with pytest.raises(cm.ValidationError, match="required"):
        m.OpticsGroup(pixel_size=1.0, voltage=300.0, defocus_u=1.0, defocus_v=1.0, astigmatism_angle=0.0)
    with pytest.raises(cm.ValidationError, match="less than or equal to 1"):
        m.OpticsGroup(label="x", pixel_size=1.0, voltage=300.0, defocus_u=1.0, defocus_v=1.0, astigmatism_angle=0.0,
                      amplitude_contrast_ratio=1.5)
    with pytest.raises(cm.ValidationError, match="Extra inputs"):
        m.OpticsGroup(label="x", pixel_size=1.0, voltage=300.0, defocus_u=1.0, defocus_v=1.0,
                      astigmatism_angle=0.0, not_a_field=1)
    og = m.OpticsGroup(label="x", pixel_size=1, voltage=300, defocus_u=1.0, defocus_v=1.0, astigmatism_angle=0.0,
                       mag_matrix=[1.0, 0.0, 0.0, 1.0])
    assert isinstance(og.pixel_size, float) and og.mag_matrix_tensor.shape == (2, 2)
    assert m.ComputationalConfigMatch(gpu_ids=[0, 1]).gpu_devices == [torch.device("cuda:0"), torch.device("cuda:1")]
    assert m.ComputationalConfigRefine(gpu_ids="cpu").gpu_devices == [torch.device("cpu")]
    assert m.ComputationalConfigRefine().backend == "batched"
    with pytest.raises(cm.ValidationError):
        m.ComputationalConfigMatch(num_cpus=0)


def test_yaml_subset_round_trip():
    text = "a: 1\nb:\n  - 0\n  - 1\nc:\n  d: null  # comment\n  e: [1, 2.5]\n  f: 'x: y'\ng: true\nh: 1.0e-3\n"
    d = cm.yaml_load(text)
    assert d == {"a": 1, "b": [0, 1], "c": {"d": None, "e": [1, 2.5], "f": "x: y"}, "g": True, "h": 1e-3}
    assert cm.yaml_load(cm.yaml_dump(d)) == d


# ---------------------------------------------------------------------------
# synthetic files for the managers
# ---------------------------------------------------------------------------


def _match_files(tmp_path, seed=4):
    cfg = sy.MatchConfig(image_shape=(256, 256), template_size=32, n_blobs=60, blob_radius=11.0, n_particles=2,
                         snr=1.0, seed=seed, out_of_plane_step=30.0, in_plane_step=30.0, plant_from_grid=True,
                         defocus=12000.0)
    wl = sy.make_match_workload(cfg, keep_image=True)
    vol, _ = sy.blob_volume(32, 60, 1.5, 11.0, seed)
    mic, tmpl = str(tmp_path / "micrograph.mrc"), str(tmp_path / "template.mrc")
    write_mrc(mic, wl.image)
    write_mrc(tmpl, vol)
    return wl, mic, tmpl


def _substituted(name, tmp_path, **subs):
    with open(os.path.join(GOLDEN, name)) as f:
        text = f.read()
    for k, v in subs.items():
        text = text.replace(f"@{k}@", v)
    out = tmp_path / name
    out.write_text(text)
    return str(out)


def test_match_manager_yaml_round_trip(tmp_path):
    _, mic, tmpl = _match_files(tmp_path)
    path = _substituted("match_template_config.yaml", tmp_path, MICROGRAPH=mic, TEMPLATE=tmpl,
                        OUT=str(tmp_path / "out"))
    mgr = m.MatchTemplateManager.from_yaml(path)
    assert mgr.optics_group.label == "synthetic" and mgr.computational_config.gpu_ids == [0]
    assert mgr.defocus_search_config.defocus_values.tolist() == [-200.0, 0.0, 200.0]
    mgr.save_config(str(tmp_path / "again.yaml"))
    mgr2 = m.MatchTemplateManager.from_yaml(str(tmp_path / "again.yaml"))
    assert mgr2.model_dump() == mgr.model_dump()
    mgr.save_config(str(tmp_path / "again.json"), mode="json")
    assert m.MatchTemplateManager.from_json(str(tmp_path / "again.json")).model_dump() == mgr.model_dump()
    kw = mgr.make_backend_core_function_kwargs()
    assert kw["image_dft"].shape == (256, 129) and kw["template_dft"].shape == (32, 32, 17)
    assert kw["ctf_filters"].shape == (1, 3, 32, 17) and kw["whitening_filter_template"].shape == (32, 17)
    with pytest.raises(cm.ValidationError, match="does not exist"):
        m.MatchTemplateManager(**{**mgr.model_dump(), "micrograph_path": str(tmp_path / "missing.mrc")})


@pytest.mark.skipif(not os.path.isdir(REF_PROGRAMS), reason="the reference's example configurations are not here")
def test_reference_example_yaml_loads(tmp_path):
    """The reference's own example configuration, with synthetic files
    substituted for its placeholder paths, loads into these managers."""
    _, mic, tmpl = _match_files(tmp_path)
    with open(os.path.join(REF_PROGRAMS, "match_template", "match_template_example_config.yaml")) as f:
        text = f.read()
    text = text.replace("/some/path/to/template.mrc", tmpl).replace("/some/path/to/micrograph.mrc", mic)
    text = text.replace("/some/path/to/", str(tmp_path / "out") + "/")
    p = tmp_path / "ref.yaml"
    p.write_text(text)
    mgr = m.MatchTemplateManager.from_yaml(str(p))
    assert mgr.optics_group.defocus_u == 5200.0 and mgr.optics_group.ctf_B_factor == 60.0
    assert mgr.defocus_search_config.defocus_values.shape == (13,)
    assert mgr.orientation_search_config.euler_angles.shape == (1584000, 3)


def test_valid_cropping(tmp_path):
    paths = {f"{k}_path": str(tmp_path / f"{k}.mrc") for k in m.MatchTemplateResult.MAPS}
    r = m.MatchTemplateResult(**paths, **{k: torch.zeros(128, 128) for k in m.MatchTemplateResult.MAPS})
    r.apply_valid_cropping((32, 32))
    assert r.mip.shape == (97, 97) and r.relative_defocus.shape == (97, 97)


def _particle_files(tmp_path, wl, mic, tmpl):
    """Particle table + statistics maps for the planted particles of ``wl``."""
    crop = 256 - 32 + 1
    avg, var = str(tmp_path / "corr_avg.mrc"), str(tmp_path / "corr_var.mrc")
    write_mrc(avg, torch.zeros(crop, crop))
    write_mrc(var, torch.ones(crop, crop))
    n = len(wl.planted)
    cols = {c: [0.0] * n for c in MATCH_TEMPLATE_DF_COLUMN_ORDER}
    for i, (y0, x0, _, eul) in enumerate(wl.planted):
        vals = dict(particle_index=i, pos_y=y0, pos_x=x0, pos_y_img=y0 + 16, pos_x_img=x0 + 16, phi=eul[0],
                    theta=eul[1], psi=eul[2], relative_defocus=0.0, defocus_u=12000.0, defocus_v=12000.0,
                    astigmatism_angle=0.0, pixel_size=1.0, refined_pixel_size=1.0, voltage=300.0,
                    spherical_aberration=2.7, amplitude_contrast_ratio=0.07, phase_shift=0.0, ctf_B_factor=0.0,
                    even_zernikes=None, odd_zernikes=None, mag_matrix=None, micrograph_path=mic,
                    template_path=tmpl, correlation_average_path=avg, correlation_variance_path=var)
        for k, v in vals.items():
            cols[k][i] = v
    for k in ("mip_path", "scaled_mip_path", "psi_path", "theta_path", "phi_path", "defocus_path"):
        cols[k] = [str(tmp_path / f"{k}.mrc")] * n
    csv_path = str(tmp_path / "particles.csv")
    write_particle_table(csv_path, cols)
    return csv_path


def test_particle_stack_and_refine_kwargs(tmp_path):
    wl, mic, tmpl = _match_files(tmp_path)
    csv_path = _particle_files(tmp_path, wl, mic, tmpl)
    path = _substituted("refine_template_config.yaml", tmp_path, TEMPLATE=tmpl, PARTICLES=csv_path)
    mgr = m.RefineTemplateManager.from_yaml(path)
    ps = mgr.particle_stack
    assert ps.num_particles == 2 and ps.extracted_box_size == (64, 64)
    with pytest.warns(UserWarning):
        eul = ps.get_euler_angles()
    assert torch.allclose(eul.float(), torch.tensor([p[3] for p in wl.planted], dtype=torch.float32))
    kw = mgr.make_backend_core_function_kwargs()
    assert kw["particle_stack_dft"].shape == (2, 64, 33) and kw["template_dft"].shape == (32, 32, 17)
    assert kw["corr_mean"].shape == (2, 33, 33) and kw["corr_std"].shape == (2, 33, 33)
    assert kw["projective_filters"].shape == (2, 32, 17)
    assert kw["euler_angle_offsets"].shape[1] == 3 and kw["defocus_offsets"].tolist() == [-100, -50, 0, 50, 100]
    assert kw["ctf_kwargs"]["pixel_size"] == 1.0 and kw["mag_matrix"] is None
    # the particle box holds the planted particle's template-corner region
    y0, x0 = wl.planted[0][:2]
    mics, idx = ps.load_images_grouped_by_column("micrograph_path")
    box = ps.construct_image_stack(mics, idx, (64, 64))
    assert torch.equal(box[0, 16:48, 16:48], wl.image[y0:y0 + 32, x0:x0 + 32]) or \
        (y0 < 16 or x0 < 16 or y0 + 48 > 256 or x0 + 48 > 256)
    bad = dict(df_path=csv_path, extracted_box_size=(32, 32), original_template_size=(32, 32))
    with pytest.raises(ValueError):
        m.ParticleStack(**bad)
    # learned proposals see a 64 x 64 band: 64-pixel crops are refused before any device work
    with pytest.raises(ValueError, match="at least 128"):
        mgr.run_refine_template_learned()


# ---------------------------------------------------------------------------
# end to end on the GPU
# ---------------------------------------------------------------------------


@pytest.mark.gpu
def test_match_manager_from_yaml_finds_planted_particles(tmp_path):
    wl, mic, tmpl = _match_files(tmp_path)
    path = _substituted("match_template_config.yaml", tmp_path, MICROGRAPH=mic, TEMPLATE=tmpl,
                        OUT=str(tmp_path / "out"))
    mgr = m.MatchTemplateManager.from_yaml(path, preload_mrc_files=True)
    mgr.run_match_template(orientation_batch_size=8, do_result_export=True)
    r = mgr.match_template_result
    assert r.mip.shape == (225, 225) and r.total_defocus == 3
    for name in m.MatchTemplateResult.MAPS:
        assert os.path.exists(getattr(r, f"{name}_path")), name
    for y0, x0, oi, eul in wl.planted:
        # the planted orientation lies on the grid: its pixel carries it
        assert (float(r.orientation_phi[y0, x0]), float(r.orientation_theta[y0, x0]),
                float(r.orientation_psi[y0, x0])) == pytest.approx(eul, abs=1e-4)
        assert float(r.relative_defocus[y0, x0]) == 0.0
    peaks = r.locate_peaks(z_score_cutoff=float(r.scaled_mip[wl.planted[0][0], wl.planted[0][1]]) - 1e-3,
                           mask_radius=5.0)
    assert bool((peaks.scaled_mip[1:] <= peaks.scaled_mip[:-1]).all())
    assert peaks.total_correlations == r.total_projections


@pytest.mark.gpu
def test_refine_manager_from_yaml_recovers_planted_poses(tmp_path):
    wl, mic, tmpl = _match_files(tmp_path)
    csv_path = _particle_files(tmp_path, wl, mic, tmpl)
    path = _substituted("refine_template_config.yaml", tmp_path, TEMPLATE=tmpl, PARTICLES=csv_path)
    mgr = m.RefineTemplateManager.from_yaml(path)
    res = mgr.run_refine_template(orientation_batch_size=16)
    assert set(res) >= {"refined_z_score", "refined_euler_angles", "refined_pos_y", "angle_idx"}
    eul = torch.as_tensor(res["refined_euler_angles"]).reshape(-1, 3)
    assert eul.shape == (2, 3)
    z = torch.as_tensor(res["refined_z_score"]).reshape(-1)
    assert bool((z > 5.0).all()), z
    # the planted poses are the starting poses: the refined rotation stays
    # inside the searched local grid (+-2 deg about two axes, at most 2.83 deg
    # from the start; a 32-voxel template is nearly flat over that range)
    from leopard_em_gb300.proposal import angular_error_deg
    from leopard_em_gb300.rotations import euler_zyz_to_rotmat

    planted = torch.tensor([p[3] for p in wl.planted], dtype=torch.float64)
    err = angular_error_deg(euler_zyz_to_rotmat(eul.double()), euler_zyz_to_rotmat(planted))
    assert float(err.max()) <= 2.0 * 2.0**0.5 + 1e-3, (eul, planted, err)
    assert np.allclose(np.asarray(res["refined_pos_y"]).reshape(-1), 0.0, atol=1.0)


@pytest.mark.gpu
def test_refine_manager_learned_proposals_run_through_the_manager(tmp_path):
    """run_refine_template_learned on 128-pixel crops: the same result keys and
    shapes as the plain grid, every particle either accepted from its proposal
    or refined by the manager's full grid, and the planted particles found."""
    wl, mic, tmpl = _match_files(tmp_path)
    csv_path = _particle_files(tmp_path, wl, mic, tmpl)
    path = _substituted("refine_template_config.yaml", tmp_path, TEMPLATE=tmpl, PARTICLES=csv_path)
    mgr = m.RefineTemplateManager.from_yaml(path)
    mgr.particle_stack.extracted_box_size = (128, 128)
    plain = mgr.run_refine_template(orientation_batch_size=16)
    for which in ("network", "gauss_newton"):
        res, info = mgr.run_refine_template_learned(orientation_batch_size=16, proposal=which)
        assert set(res) == set(plain) and info["particles"] == 2 and 0 <= info["fallback"] <= 2
        for k, v in plain.items():
            if isinstance(v, torch.Tensor):
                assert tuple(torch.as_tensor(res[k]).shape) == tuple(v.shape), k
        z = torch.as_tensor(res["refined_z_score"]).reshape(-1)
        assert bool((z > 5.0).all()), (which, z)
