"""GPU parity of the local-grid refinement (core_refine_template) through the C ABI.

Against the golden vectors recorded from the reference's own
_core_refine_template_single_thread, and against the CPU oracle at larger
sizes (including a 288^2 crop).  Acceptance: winning offsets, defocus and
pixel-size offsets, position and angle index identical; refined z-score and
cross-correlation within 1e-4 relative (of max(|value|, 1)).
"""

import os

import numpy as np
import pytest
import torch

from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300.backend import core_refine_template
from oracle import ref_refine_template as orr

pytestmark = pytest.mark.gpu
RTOL = 1e-4
RGOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "refine_small.npz"))


def _golden_kwargs():
    keys = ["particle_stack_dft", "template_dft", "euler_angles", "euler_angle_offsets", "defocus_offsets",
            "pixel_size_offsets", "defocus_u", "defocus_v", "defocus_angle", "corr_mean", "corr_std",
            "projective_filters"]
    kw = {k: torch.from_numpy(RGOLD[f"in/{k}"]) for k in keys}
    ctf = {k.split("/", 1)[1]: RGOLD[k].item() for k in RGOLD.files if k.startswith("ctf/")}
    d = kw["template_dft"].shape[1]
    ctf.update(template_shape=(d, d), even_zernikes=None, odd_zernikes=None, mag_matrix=None)
    kw["ctf_kwargs"] = ctf
    return kw, int(RGOLD["in/batch_size"])


def _close(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.all(np.abs(a - b) <= RTOL * np.maximum(np.abs(b), 1.0))


def test_refine_against_reference_golden_vectors():
    kw, b = _golden_kwargs()
    res = core_refine_template(**kw, device=torch.device("cuda:0"), batch_size=b)
    g = {k[4:]: RGOLD[k] for k in RGOLD.files if k.startswith("out/")}
    assert _close(res["refined_z_score"].numpy(), g["max_z_score"])
    assert _close(res["refined_cross_correlation"].numpy(), g["max_cc"])
    H, d = kw["particle_stack_dft"].shape[1], kw["template_dft"].shape[1]
    off = (H - d + 1) // 2
    assert np.array_equal(res["refined_pos_y"].numpy() + off, g["refined_pos_y"].astype(np.int64))
    assert np.array_equal(res["refined_pos_x"].numpy() + off, g["refined_pos_x"].astype(np.int64))
    assert np.array_equal(res["angle_idx"].numpy(), g["angle_idx"].astype(np.int64))
    assert np.array_equal(res["refined_defocus_offset"].numpy(), g["refined_defocus_offset"].astype(np.float32))
    assert np.array_equal(res["refined_pixel_size_offset"].numpy(),
                          g["refined_pixel_size_offset"].astype(np.float32))


def _synthetic_refine(n_p, H, d, n_off, D, C, seed):
    g = torch.Generator().manual_seed(seed)
    vol, _ = sy.blob_volume(d, 80, 1.5, d * 0.3, seed)
    from leopard_em_gb300 import preprocess as pp

    template_dft = pp.volume_to_rfft_fourier_slice(vol).to(torch.complex64)
    stack = []
    for _ in range(n_p):
        f = torch.fft.rfftn(torch.randn(H, H, generator=g))
        f[0, 0] = 0
        stack.append(f / torch.sqrt((f.abs() ** 2).sum() * 2) * H)
    crop = H - d + 1
    offs = (torch.rand(n_off, 3, generator=g) - 0.5) * 6.0
    offs[0] = 0
    return dict(
        particle_stack_dft=torch.stack(stack).to(torch.complex64), template_dft=template_dft,
        euler_angles=torch.rand(n_p, 3, generator=g) * torch.tensor([360.0, 180.0, 360.0]),
        euler_angle_offsets=offs, defocus_offsets=torch.linspace(-200, 200, D),
        defocus_u=8000 + 4000 * torch.rand(n_p, generator=g), defocus_v=8000 + 4000 * torch.rand(n_p, generator=g),
        defocus_angle=90 * torch.rand(n_p, generator=g),
        pixel_size_offsets=torch.linspace(-0.02, 0.02, C) if C > 1 else torch.zeros(1),
        corr_mean=0.05 * torch.randn(n_p, crop, crop, generator=g),
        corr_std=0.8 + 0.4 * torch.rand(n_p, crop, crop, generator=g),
        ctf_kwargs=dict(voltage=300.0, spherical_aberration=2.7, amplitude_contrast_ratio=0.07, ctf_B_factor=80.0,
                        phase_shift=0.0, pixel_size=1.06, template_shape=(d, d), even_zernikes=None,
                        odd_zernikes=None, mag_matrix=None),
        projective_filters=torch.ones(n_p, d, d // 2 + 1),
    )


@pytest.mark.parametrize("n_p,H,d,n_off,D,C,batch", [(3, 128, 64, 10, 3, 2, 4), (2, 288, 256, 5, 2, 1, 3)])
def test_refine_against_oracle(n_p, H, d, n_off, D, C, batch):
    kw = _synthetic_refine(n_p, H, d, n_off, D, C, seed=H + n_off)
    ref = orr.core_refine_template_cpu(**kw, batch_size=batch)
    got = core_refine_template(**kw, device=torch.device("cuda:0"), batch_size=batch)
    assert _close(got["refined_z_score"].numpy(), ref["refined_z_score"].numpy())
    assert _close(got["refined_cross_correlation"].numpy(), ref["refined_cross_correlation"].numpy())
    for k in ["refined_pos_y", "refined_pos_x", "angle_idx"]:
        assert np.array_equal(got[k].numpy(), ref[k].numpy()), k
    for k in ["refined_defocus_offset", "refined_pixel_size_offset"]:
        assert np.array_equal(got[k].numpy(), ref[k].numpy().astype(np.float32)), k
    assert np.allclose(got["refined_euler_angles"].numpy(), ref["refined_euler_angles"].numpy(), atol=1e-3)
    assert set(got) == {"refined_cross_correlation", "refined_z_score", "refined_euler_angles",
                        "refined_defocus_offset", "refined_pixel_size_offset", "refined_pos_y", "refined_pos_x",
                        "angle_idx"}


def test_refine_particle_groups_match_single_call():
    """Splitting the stack into several device calls gives the same answers."""
    from leopard_em_gb300.backend.core_refine_template import refine_particles_device

    kw = _synthetic_refine(5, 128, 64, 6, 2, 1, seed=9)
    a = refine_particles_device(**kw, device=torch.device("cuda:0"), batch_size=4)
    b = refine_particles_device(**kw, device=torch.device("cuda:0"), batch_size=4, max_correlograms_per_call=16)
    for k in a:
        assert torch.equal(a[k], b[k]), k


def test_learned_proposals_match_plain_grid_snr_with_fewer_correlations():
    """Shipped network on 128 particles of the production refinement
    configuration, each run through both methods: the proposal + small grid
    (+ full-grid fallback) reaches a mean refined SNR at least the plain full
    grid's (no slack) while computing far fewer correlograms.  Ablation: the
    Gauss-Newton step alone (the network's own input channels, no network)
    through the same verification and fallback; the network must need no more
    full-grid fallbacks than it."""
    from leopard_em_gb300 import proposal as pr

    path = os.path.join(os.path.dirname(os.path.dirname(__file__)), "leopard_em_gb300", "weights",
                        "proposal_refine288.npz")
    cfg = sy.CONFIG_REFINE
    dev = torch.device("cuda:0")
    kw, _ = sy.make_refine_workload(cfg, 128, device=dev, seed_offset=777)
    plain = core_refine_template(**kw, device=dev, batch_size=cfg.batch)
    net = pr.load_net(path, dev)
    small = sy.local_euler_offsets(0.5, 0.125, 0.5, 0.125)
    small_df = torch.arange(-100.0, 100.0 + 1e-6, 50.0)
    res, info = pr.refine_with_proposals(net, kw, dev, small, small_df, batch_size=cfg.batch)
    res_gn, info_gn = pr.refine_with_proposals(None, kw, dev, small, small_df, batch_size=cfg.batch,
                                               proposal="gauss_newton")
    zp = plain["refined_z_score"].double().mean().item()
    zl = res["refined_z_score"].double().mean().item()
    zg = res_gn["refined_z_score"].double().mean().item()
    print(f"mean refined SNR over 128 particles: plain {zp:.4f} learned {zl:.4f} gauss-newton only {zg:.4f}; "
          f"fallbacks learned {info['fallback']} gauss-newton {info_gn['fallback']}; correlograms/particle "
          f"{info['correlations_per_particle']:.0f} (gauss-newton {info_gn['correlations_per_particle']:.0f}) "
          f"vs {info['full_grid_correlations']}")
    assert zl >= zp
    assert info["correlations_per_particle"] < info["full_grid_correlations"] / 5
    assert info["fallback"] <= info_gn["fallback"]