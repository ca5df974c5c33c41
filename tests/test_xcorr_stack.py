"""cross_correlate_particle_stack (core_refine_template.py:771-895): the oracle
against vectors recorded from the reference's own function (CPU), the device
path against both (GPU).  Tolerance: 1e-4 of the largest |correlation| (FP32
FFTs of different factorisations)."""

import os

import numpy as np
import pytest
import torch

from oracle import ref_refine_template as orr

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "xcorr_small.npz"))


def _case(name):
    return (torch.from_numpy(GOLD[f"{name}/stack"]), torch.from_numpy(GOLD[f"{name}/template_dft"]),
            torch.from_numpy(GOLD[f"{name}/rot"]), torch.from_numpy(GOLD[f"{name}/filters"]))


def _close(got, ref, tol=1e-4):
    ref = np.asarray(ref)
    err = np.abs(np.asarray(got) - ref).max() / np.abs(ref).max()
    assert err <= tol, f"relative error {err:.3e}"


@pytest.mark.parametrize("name", ["x1", "x2"])
@pytest.mark.parametrize("mode", ["valid", "same"])
def test_oracle_matches_reference(name, mode):
    got = orr.cross_correlate_particle_stack_cpu(*_case(name), mode=mode)
    _close(got.numpy(), GOLD[f"{name}/{mode}"], 1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["x1", "x2"])
@pytest.mark.parametrize("mode", ["valid", "same"])
@pytest.mark.parametrize("batch", [1, 2, -1])
def test_device_matches_reference(name, mode, batch):
    from leopard_em_gb300.backend import cross_correlate_particle_stack

    got = cross_correlate_particle_stack(*_case(name), mode=mode, batch_size=batch)
    assert got.device.type == "cpu" and tuple(got.shape) == GOLD[f"{name}/{mode}"].shape
    _close(got.numpy(), GOLD[f"{name}/{mode}"])


@pytest.mark.gpu
def test_device_matches_oracle_refine_size():
    """288^2 crops with a 256^3 template (the refinement configuration's shapes)."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.backend import cross_correlate_particle_stack

    cfg = sy.RefineConfig(crop=288, template_size=256, n_blobs=300, blob_radius=80.0)
    kw, _ = sy.make_refine_workload(cfg, 3)
    rot = sy.axis_angle_rotations(torch.tensor([[0.0, 0.0, 1.0]] * 3), torch.tensor([0.1, 0.7, 2.0]))
    pf = kw["projective_filters"]
    ps = kw["particle_stack_dft"].clone()
    ps[:, 0, 0] = 5.0 + 0j  # non-zero DC: the term the search path zeroes
    got = cross_correlate_particle_stack(ps.cuda(), kw["template_dft"], rot.float(), pf, mode="valid")
    assert got.is_cuda
    ref = orr.cross_correlate_particle_stack_cpu(ps, kw["template_dft"], rot.float(), pf, mode="valid")
    _close(got.cpu().numpy(), ref.numpy())


@pytest.mark.gpu
def test_device_argument_errors():
    from leopard_em_gb300.backend import cross_correlate_particle_stack

    ps, t, r, f = _case("x1")
    with pytest.raises(ValueError):
        cross_correlate_particle_stack(ps, t, r, f, mode="full")
    with pytest.raises(ValueError):
        cross_correlate_particle_stack(ps, t, r[:2], f)
    with pytest.raises(ValueError):
        cross_correlate_particle_stack(ps, t, r, f, mag_matrix=torch.eye(2))
