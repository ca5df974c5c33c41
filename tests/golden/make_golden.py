"""Generate golden vectors for the 2DTM search by running the reference's own code.

Run once, in a container that holds the Leopard-EM source tree (read-only):

    python tests/golden/make_golden.py /root/reference

It imports, straight from the source files,
``src/leopard_em/backend/cross_correlation.py``, ``backend/utils.py`` and
``backend/process_results.py``.  Their third-party imports ``roma`` and
``torch_fourier_slice`` are not installed, so two stand-in modules are
registered in ``sys.modules`` that delegate to the oracle's restatements
(``euler_to_rotmat_zyz``, ``extract_central_slices_rfft_3d``).  Everything else
-- filter application, irfft2, ifftshift, projection normalisation, padded
forward FFT, cross-power, irfft2, MIP/argmax/sum updates, index decoding and
z-score scaling -- is the reference's own code, driven by the orientation loop
of ``backend/core_match_template.py:492-550`` (which itself needs CUDA streams
and is therefore restated in this script's ``_run_search``).

Outputs ``tests/golden/match_small.npz``: inputs and outputs of two small
searches (one with several defocus planes and pixel sizes, run with the
reference's batched CPU path and per-batch statistics update).  The files are
small (< 1 MB) and committed; this script is not needed at test time.
"""

from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import ref_match_template as orc  # noqa: E402


def _install_stubs():
    roma = types.ModuleType("roma")

    def euler_to_rotmat(convention, angles, degrees=True, device=None, **_):
        assert convention == "ZYZ" and degrees
        return orc.euler_to_rotmat_zyz(torch.as_tensor(angles), dtype=torch.float32)

    roma.euler_to_rotmat = euler_to_rotmat
    roma.rotmat_composition = lambda seq: seq[0] @ seq[1]
    sys.modules["roma"] = roma

    tfs = types.ModuleType("torch_fourier_slice")
    tfs.extract_central_slices_rfft_3d = (
        lambda volume_rfft, rotation_matrices, **_: orc.extract_central_slices_rfft_3d(volume_rfft, rotation_matrices)
    )

    def _no_mag(*a, **k):
        raise NotImplementedError("anisotropic magnification is not used by the golden cases")

    tfs.transform_slice_2d = _no_mag
    sys.modules["torch_fourier_slice"] = tfs


def _load(ref_root, rel, name):
    path = os.path.join(ref_root, "src", "leopard_em", *rel.split("/"))
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def _make_inputs(seed, H, W, d, n_o, n_df, n_cs):
    g = torch.Generator().manual_seed(seed)
    image = torch.randn(H, W, generator=g, dtype=torch.float32)
    image_dft = torch.fft.rfftn(image)
    image_dft[0, 0] = 0
    image_dft = image_dft / torch.sqrt((image_dft.abs() ** 2).sum() * 2)
    image_dft = image_dft * (H * W) ** 0.5
    # smooth random template
    vol = torch.randn(d, d, d, generator=g, dtype=torch.float32)
    kern = torch.exp(-torch.arange(-3, 4, dtype=torch.float32) ** 2 / 4.0)
    kern = kern / kern.sum()
    for ax in range(3):
        vol = torch.nn.functional.conv1d(
            vol.movedim(ax, -1).reshape(-1, 1, d), kern.view(1, 1, -1), padding=3
        ).reshape(*[d] * 3).movedim(-1, ax)
    template_dft = orc.volume_to_rfft_fourier_slice(vol)
    wc = d // 2 + 1
    ky = torch.fft.fftfreq(d)[:, None]
    kx = torch.fft.rfftfreq(d)[None, :]
    k2 = ky**2 + kx**2
    dfs = torch.linspace(-0.4, 0.4, n_df)
    ctf = torch.stack(
        [torch.stack([-torch.sin(6.0 * (1.0 + c * 0.1 + df) * k2 * 40 + 0.07) for df in dfs]) for c in range(n_cs)]
    ).to(torch.float32)
    whitening = (1.0 / (1.0 + 3.0 * k2)).to(torch.float32)
    assert ctf.shape == (n_cs, n_df, d, wc)
    euler = torch.rand(n_o, 3, generator=g) * torch.tensor([360.0, 180.0, 360.0])
    defocus_values = torch.linspace(-200.0, 200.0, n_df)
    pixel_values = torch.linspace(-0.02, 0.02, n_cs) if n_cs > 1 else torch.zeros(1)
    return dict(
        image_dft=image_dft, template_dft=template_dft, ctf_filters=ctf,
        whitening_filter_template=whitening, defocus_values=defocus_values,
        pixel_values=pixel_values, euler_angles=euler.to(torch.float32),
    )


def _run_search(cc_mod, ut_mod, pr_mod, inp, batch):
    """Orientation loop of core_match_template.py:492-550 on the CPU."""
    image_dft, template_dft = inp["image_dft"], inp["template_dft"]
    pf = inp["ctf_filters"] * inp["whitening_filter_template"][None, None, ...]
    euler = inp["euler_angles"]
    dfv, pxv = inp["defocus_values"], inp["pixel_values"]
    n_o, n_df, n_cs = euler.shape[0], dfv.shape[0], pxv.shape[0]
    assert n_o % batch == 0
    H, W = image_dft.shape[0], image_dft.shape[1] * 2 - 2
    incr = torch.tensor([df * n_o + cs * n_df * n_o for cs in range(n_cs) for df in range(n_df)], dtype=torch.int32)
    mip = torch.full((H, W), -float("inf"))
    best = torch.full((H, W), -1, dtype=torch.int32)
    s1 = torch.zeros((H, W))
    s2 = torch.zeros((H, W))
    for i in range(0, n_o, batch):
        rot = sys.modules["roma"].euler_to_rotmat("ZYZ", euler[i : i + batch], degrees=True)
        idx = torch.arange(i, i + batch, dtype=torch.int32)
        bsi = (idx + incr[:, None]).flatten()
        cc = cc_mod.do_batched_orientation_cross_correlate_cpu(
            image_dft=image_dft, template_dft=template_dft, rotation_matrices=rot, projective_filters=pf
        )
        ut_mod.do_iteration_statistics_updates(cc, bsi, mip, best, s1, s2, H, W)
    phi, theta, psi, defocus = pr_mod.decode_global_search_index(best, pxv, dfv, euler)
    total = n_o * n_df * n_cs
    mip, scaled, mean, std = pr_mod.scale_mip(mip, torch.empty_like(mip), s1, s2, total)
    return dict(
        mip=mip, scaled_mip=scaled, best_phi=phi, best_theta=theta, best_psi=psi, best_defocus=defocus,
        correlation_mean=mean, correlation_variance=std, best_global_index=best,
    )


def main(ref_root):
    os.environ["LEOPARDEM_DISABLE_TORCH_COMPILATION"] = "1"
    _install_stubs()
    ut = _load(ref_root, "backend/utils.py", "leopard_em_ref_utils")
    sys.modules["leopard_em.backend.utils"] = ut
    sys.modules.setdefault("leopard_em", types.ModuleType("leopard_em"))
    sys.modules.setdefault("leopard_em.backend", types.ModuleType("leopard_em.backend"))
    cc = _load(ref_root, "backend/cross_correlation.py", "leopard_em_ref_cc")
    pr = _load(ref_root, "backend/process_results.py", "leopard_em_ref_pr")

    out = {}
    cases = {
        "a": dict(seed=11, H=64, W=64, d=16, n_o=8, n_df=2, n_cs=1, batch=4),
        "b": dict(seed=12, H=48, W=80, d=16, n_o=6, n_df=3, n_cs=2, batch=3),
    }
    for name, c in cases.items():
        inp = _make_inputs(c["seed"], c["H"], c["W"], c["d"], c["n_o"], c["n_df"], c["n_cs"])
        res = _run_search(cc, ut, pr, inp, c["batch"])
        # single-batch correlogram and normalised projection straight from the reference
        rot = sys.modules["roma"].euler_to_rotmat("ZYZ", inp["euler_angles"][: c["batch"]], degrees=True)
        pf = inp["ctf_filters"] * inp["whitening_filter_template"][None, None, ...]
        ccv = cc.do_batched_orientation_cross_correlate_cpu(inp["image_dft"], inp["template_dft"], rot, pf)
        out[f"{name}/batch"] = np.array(c["batch"])
        out[f"{name}/cc_first_batch"] = ccv.numpy()
        for k, v in inp.items():
            out[f"{name}/in/{k}"] = v.numpy()
        for k, v in res.items():
            out[f"{name}/out/{k}"] = v.numpy()
    # normalisation kernel alone (utils.py:106-188)
    g = torch.Generator().manual_seed(5)
    p = torch.randn(3, 20, 20, generator=g) + 0.3
    out["norm/in"] = p.numpy()
    out["norm/out"] = ut.normalize_template_projection(p, (20, 20), (64, 96)).numpy()
    # results epilogue alone (process_results.py)
    gi = torch.randint(0, 2 * 3 * 5, (7, 9), generator=g, dtype=torch.int32)
    eul = torch.rand(5, 3, generator=g) * 360
    dfv = torch.tensor([-100.0, 0.0, 100.0])
    phi, theta, psi, dd = pr.decode_global_search_index(gi, torch.zeros(2), dfv, eul)
    out["decode/gi"] = gi.numpy()
    out["decode/euler"] = eul.numpy()
    out["decode/defocus"] = dfv.numpy()
    out["decode/out"] = torch.stack([phi, theta, psi, dd]).numpy()
    path = os.path.join(HERE, "match_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
