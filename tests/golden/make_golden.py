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
reference's batched CPU path and per-batch statistics update).

``tests/golden/refine_small.npz``: per-particle results of the reference's
``_core_refine_template_single_thread`` (backend/core_refine_template.py:555-767,
its CPU branch), with roma / torch_fourier_slice / torch_ctf /
torch_fourier_filter replaced by the oracle's restatements
(``oracle/ref_refine_template.py``) and the rest -- ctf_utils.py,
search_utils.py, the cross-correlation, z-score, strict-'>' batch update and
index decode -- the reference's own code.

``tests/golden/peaks_small.npz`` (``--peaks``): z-score peak picking by the
reference's ``analysis/zscore_metric.py`` (find_peaks_from_zscore,
gaussian_noise_zscore_cutoff) and ``analysis/utils.py``
(filter_peaks_by_distance); ``pandas`` (imported by the package's
match_template_peaks.py, unused here) is a stand-in module.

``tests/golden/preprocess_small.npz`` (``--preprocess``): the reference's
``preprocess_image`` (utils/image_processing.py:16-75) and its CTF-stack
wrapper (utils/ctf_utils.py:19-116) with the stand-ins above for torch_ctf.

``tests/golden/xcorr_small.npz`` (``--xcorr``): the reference's
``cross_correlate_particle_stack`` (backend/core_refine_template.py:771-895)
on small stacks, both modes, with the stand-ins above for the slice extraction.

The files are small and committed; this script is not needed at test time.
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
from oracle import ref_refine_template as orr  # noqa: E402


def _install_stubs():
    roma = types.ModuleType("roma")

    def euler_to_rotmat(convention, angles, degrees=True, device=None, **_):
        assert convention == "ZYZ" and degrees
        return orc.euler_to_rotmat_zyz(torch.as_tensor(angles), dtype=torch.float32)

    roma.euler_to_rotmat = euler_to_rotmat
    roma.rotmat_composition = lambda seq: seq[0] @ seq[1]
    roma.rotmat_to_euler = lambda convention, R, degrees=True, **_: orr.rotmat_to_euler_zyz(R).to(R.dtype)
    sys.modules["roma"] = roma

    tctf = types.ModuleType("torch_ctf")

    def calculate_ctf_2d(defocus, astigmatism, astigmatism_angle, voltage, spherical_aberration, amplitude_contrast,
                         phase_shift, pixel_size, image_shape, rfft=True, fftshift=False, even_zernike_coeffs=None,
                         odd_zernike_coeffs=None, transform_matrix=None):
        assert rfft and not fftshift and even_zernike_coeffs is None and odd_zernike_coeffs is None
        assert transform_matrix is None
        return orr.calculate_ctf_2d(defocus, astigmatism, astigmatism_angle, voltage, float(spherical_aberration),
                                    amplitude_contrast, phase_shift, pixel_size, tuple(image_shape))

    tctf.calculate_ctf_2d = calculate_ctf_2d
    sys.modules["torch_ctf"] = tctf
    tff = types.ModuleType("torch_fourier_filter")
    env = types.ModuleType("torch_fourier_filter.envelopes")
    env.b_envelope = lambda B, image_shape, pixel_size, rfft=True, fftshift=False, device=None: orr.b_envelope(
        B, tuple(image_shape), pixel_size)
    tff.envelopes = env
    sys.modules["torch_fourier_filter"] = tff
    sys.modules["torch_fourier_filter.envelopes"] = env

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


def _peak_maps():
    """Seeded z maps: N(0,1) noise plus Gaussian bumps (no exact ties)."""
    g = torch.Generator().manual_seed(21)
    maps = {}
    for name, (H, W, n_bumps, amp) in {"p1": (64, 80, 6, 10.0), "p2": (96, 96, 25, 7.0), "p3": (40, 40, 0, 0.0)}.items():
        z = torch.randn(H, W, generator=g)
        yy, xx = torch.meshgrid(torch.arange(H, dtype=torch.float32), torch.arange(W, dtype=torch.float32),
                                indexing="ij")
        for _ in range(n_bumps):
            cy, cx = (torch.rand(2, generator=g) * torch.tensor([H - 1.0, W - 1.0])).tolist()
            sig = 1.0 + 2.0 * torch.rand(1, generator=g).item()
            z += amp * torch.rand(1, generator=g).item() * torch.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * sig**2))
        maps[name] = z
    return maps


def main_peaks(ref_root):
    pd = types.ModuleType("pandas")
    pd.DataFrame = dict  # only named in an annotation
    sys.modules.setdefault("pandas", pd)
    pkg = types.ModuleType("leopard_em_ref_analysis")
    pkg.__path__ = [os.path.join(ref_root, "src/leopard_em/analysis")]
    sys.modules["leopard_em_ref_analysis"] = pkg
    mods = {}
    for sub in ("match_template_peaks", "utils", "zscore_metric"):
        path = os.path.join(ref_root, "src/leopard_em/analysis", sub + ".py")
        spec = importlib.util.spec_from_file_location(f"leopard_em_ref_analysis.{sub}", path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[f"leopard_em_ref_analysis.{sub}"] = mod
        spec.loader.exec_module(mod)
        mods[sub] = mod
    zm = mods["zscore_metric"]
    out = {}
    for name, z in _peak_maps().items():
        for cutoff, radius in ((3.0, 5.0), (2.0, 2.5), (4.0, 10.0)):
            py, px = zm.find_peaks_from_zscore(z, cutoff, radius)
            key = f"{name}/c{cutoff}/r{radius}"
            out[f"{key}/pos_y"] = py.numpy()
            out[f"{key}/pos_x"] = px.numpy()
        out[f"{name}/z"] = z.numpy()
    n_ccg = np.array([10**6, 10**9, 4096 * 4096 * 1584000 * 3], dtype=np.float64)
    out["cutoff/num_ccg"] = n_ccg
    out["cutoff/value"] = np.array([zm.gaussian_noise_zscore_cutoff(int(n), fp) for n in n_ccg for fp in (1.0, 0.5)])
    np.savez_compressed(os.path.join(HERE, "peaks_small.npz"), **out)


def main_xcorr(ref_root):
    """cross_correlate_particle_stack (core_refine_template.py:771-895) from the
    reference's own code -> xcorr_small.npz (particles with a non-zero DC)."""
    os.environ["LEOPARDEM_DISABLE_TORCH_COMPILATION"] = "1"
    _install_stubs()
    ut = _load(ref_root, "backend/utils.py", "leopard_em_ref_utils")
    sys.modules["leopard_em.backend.utils"] = ut
    sys.modules.setdefault("leopard_em", types.ModuleType("leopard_em"))
    sys.modules.setdefault("leopard_em.backend", types.ModuleType("leopard_em.backend"))
    _load(ref_root, "backend/cross_correlation.py", "leopard_em_ref_cc")
    for name in ("leopard_em.utils",):
        sys.modules.setdefault(name, types.ModuleType(name))
    _load(ref_root, "utils/search_utils.py", "leopard_em.utils.search_utils")
    _load(ref_root, "utils/cross_correlation.py", "leopard_em.utils.cross_correlation")
    _load(ref_root, "utils/ctf_utils.py", "leopard_em.utils.ctf_utils")
    _load(ref_root, "backend/distributed.py", "leopard_em.backend.distributed")
    sys.modules["leopard_em.backend.cross_correlation"] = sys.modules["leopard_em_ref_cc"]
    rt = _load(ref_root, "backend/core_refine_template.py", "leopard_em_ref_refine")
    g = torch.Generator().manual_seed(41)
    out = {}
    for name, (n_p, H, d) in {"x1": (3, 64, 32), "x2": (2, 128, 64)}.items():
        inp = _make_inputs(41 + H, H, H, d, 1, 1, 1)
        stack = torch.fft.rfftn(torch.randn(n_p, H, H, generator=g) + 0.3, dim=(-2, -1)).to(torch.complex64)
        euler = (torch.rand(n_p, 3, generator=g) * torch.tensor([360.0, 180.0, 360.0])).to(torch.float32)
        rot = sys.modules["roma"].euler_to_rotmat("ZYZ", euler, degrees=True)
        pf = (torch.rand(n_p, d, d // 2 + 1, generator=g) + 0.5).to(torch.float32)
        for mode in ("valid", "same"):
            cc = rt.cross_correlate_particle_stack(stack, inp["template_dft"], rot, pf, mode=mode, batch_size=2)
            out[f"{name}/{mode}"] = cc.numpy()
        out[f"{name}/stack"] = stack.numpy()
        out[f"{name}/template_dft"] = inp["template_dft"].numpy()
        out[f"{name}/rot"] = rot.numpy()
        out[f"{name}/filters"] = pf.numpy()
    np.savez_compressed(os.path.join(HERE, "xcorr_small.npz"), **out)


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
    _refine_golden(ref_root)


def _refine_golden(ref_root):
    for name in ("leopard_em.utils",):
        sys.modules.setdefault(name, types.ModuleType(name))
    su = _load(ref_root, "utils/search_utils.py", "leopard_em.utils.search_utils")
    _load(ref_root, "utils/cross_correlation.py", "leopard_em.utils.cross_correlation")
    _load(ref_root, "utils/ctf_utils.py", "leopard_em.utils.ctf_utils")
    _load(ref_root, "backend/distributed.py", "leopard_em.backend.distributed")
    sys.modules["leopard_em.backend.cross_correlation"] = sys.modules["leopard_em_ref_cc"]
    rt = _load(ref_root, "backend/core_refine_template.py", "leopard_em_ref_refine")
    assert su.get_cs_range is not None
    g = torch.Generator().manual_seed(31)
    n_p, H, d = 3, 48, 32
    wc = d // 2 + 1
    inp = _make_inputs(31, H, H, d, 1, 1, 1)
    template_dft = inp["template_dft"]
    stack = []
    for _ in range(n_p):
        im = torch.randn(H, H, generator=g)
        f = torch.fft.rfftn(im)
        f[0, 0] = 0
        f = f / torch.sqrt((f.abs() ** 2).sum() * 2) * (H * H) ** 0.5
        stack.append(f)
    particle_stack_dft = torch.stack(stack).to(torch.complex64)
    euler = (torch.rand(n_p, 3, generator=g) * torch.tensor([360.0, 180.0, 360.0])).to(torch.float32)
    offsets = torch.tensor([[0.0, 0.0, 0.0], [2.0, 0.0, -2.0], [-2.0, 1.5, 0.0], [0.0, -1.5, 2.0],
                            [1.0, 1.0, 1.0], [-1.0, -1.0, 3.0]], dtype=torch.float32)
    defocus_offsets = torch.tensor([-100.0, 0.0, 100.0])
    pixel_offsets = torch.tensor([-0.01, 0.01])
    du = torch.tensor([9000.0, 10000.0, 11000.0])
    dv = du - 150.0
    dang = torch.tensor([10.0, 35.0, 80.0])
    crop = H - d + 1
    corr_mean = 0.05 * torch.randn(n_p, crop, crop, generator=g)
    corr_std = 0.8 + 0.4 * torch.rand(n_p, crop, crop, generator=g)
    pf = (1.0 / (1.0 + 2.0 * torch.fft.rfftfreq(d)[None, :] ** 2 + torch.fft.fftfreq(d)[:, None] ** 2)).expand(
        n_p, d, wc).contiguous().to(torch.float32)
    ctf_kwargs = dict(voltage=300.0, spherical_aberration=2.7, amplitude_contrast_ratio=0.07, ctf_B_factor=60.0,
                      phase_shift=0.0, pixel_size=1.0, template_shape=(d, d), even_zernikes=None,
                      odd_zernikes=None, mag_matrix=None)
    keys = ["max_cc", "max_z_score", "refined_phi_offset", "refined_theta_offset", "refined_psi_offset",
            "refined_defocus_offset", "refined_pixel_size_offset", "refined_pos_y", "refined_pos_x", "angle_idx"]
    res = {k: [] for k in keys}
    for i in range(n_p):
        st = rt._core_refine_template_single_thread(
            particle_image_dft=particle_stack_dft[i], particle_index=i, template_dft=template_dft,
            euler_angles=euler[i], euler_angle_offsets=offsets, defocus_u=float(du[i]), defocus_v=float(dv[i]),
            defocus_angle=float(dang[i]), defocus_offsets=defocus_offsets, pixel_size_offsets=pixel_offsets,
            corr_mean=corr_mean[i], corr_std=corr_std[i], ctf_kwargs=ctf_kwargs, projective_filter=pf[i],
            batch_size=4)
        for k in keys:
            res[k].append(float(st[k]))
    out = {
        "in/particle_stack_dft": particle_stack_dft.numpy(), "in/template_dft": template_dft.numpy(),
        "in/euler_angles": euler.numpy(), "in/euler_angle_offsets": offsets.numpy(),
        "in/defocus_offsets": defocus_offsets.numpy(), "in/pixel_size_offsets": pixel_offsets.numpy(),
        "in/defocus_u": du.numpy(), "in/defocus_v": dv.numpy(), "in/defocus_angle": dang.numpy(),
        "in/corr_mean": corr_mean.numpy(), "in/corr_std": corr_std.numpy(), "in/projective_filters": pf.numpy(),
        "in/batch_size": np.array(4),
    }
    for k, v in ctf_kwargs.items():
        if k != "template_shape" and v is not None:
            out[f"ctf/{k}"] = np.array(v)
    for k in keys:
        out[f"out/{k}"] = np.array(res[k])
    path = os.path.join(HERE, "refine_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def main_preprocess(ref_root):
    """preprocess_image (utils/image_processing.py:16-75) and the CTF-stack
    wrapper calculate_ctf_filter_stack_full_args (utils/ctf_utils.py:19-116)
    from the reference's own code -> preprocess_small.npz.  torch_ctf /
    b_envelope are the stand-ins above (the oracle's restatements), so the CTF
    case pins the wrapper's defocus / astigmatism / Cs / envelope handling."""
    _install_stubs()
    dw = types.ModuleType("torch_fourier_filter.dose_weight")

    def _no_dose(*a, **k):
        raise NotImplementedError("dose weighting is not used by the golden cases")

    dw.dose_weight_movie = _no_dose
    sys.modules["torch_fourier_filter.dose_weight"] = dw
    for name in ("leopard_em", "leopard_em.utils"):
        sys.modules.setdefault(name, types.ModuleType(name))
    _load(ref_root, "utils/search_utils.py", "leopard_em.utils.search_utils")
    ip = _load(ref_root, "utils/image_processing.py", "leopard_em_ref_image_processing")
    cu = _load(ref_root, "utils/ctf_utils.py", "leopard_em_ref_ctf_utils")
    g = torch.Generator().manual_seed(77)
    out = {}
    # one micrograph-like spectrum, filter and bandpass
    img = torch.fft.rfftn(torch.randn(96, 128, generator=g))
    img[0, 0] = 0
    filt = (torch.rand(96, 65, generator=g) + 0.25).to(torch.float32)
    band = (torch.rand(96, 65, generator=g) > 0.2).to(torch.float32)
    out["single/image_dft"] = img.numpy()
    out["single/filter"] = filt.numpy()
    out["single/bandpass"] = band.numpy()
    out["single/out"] = ip.preprocess_image(img, filt, band, (96, 128), (96, 128)).numpy()
    # a particle stack: per-image filters, box area smaller than the image's
    stack = torch.fft.rfftn(torch.randn(3, 64, 64, generator=g), dim=(-2, -1))
    filts = (torch.rand(3, 64, 33, generator=g) + 0.1).to(torch.float32)
    band2 = torch.ones(64, 33)
    out["stack/image_dft"] = stack.numpy()
    out["stack/filter"] = filts.numpy()
    out["stack/bandpass"] = band2.numpy()
    out["stack/out"] = ip.preprocess_image(stack, filts, band2, (64, 64), (49, 49)).numpy()
    # CTF filter stack: astigmatic, B envelope, two pixel sizes, three defocus planes
    kw = dict(astigmatism_angle=25.0, voltage=300.0, spherical_aberration=2.7, amplitude_contrast_ratio=0.07,
              ctf_B_factor=60.0, phase_shift=0.0, pixel_size=1.06, even_zernikes=None, odd_zernikes=None,
              mag_matrix=None)
    dfo = torch.tensor([-200.0, 0.0, 200.0])
    pxo = torch.tensor([-0.02, 0.02])
    ctf = cu.calculate_ctf_filter_stack_full_args((32, 32), 5200.0, 4950.0, dfo, pxo, **kw)
    out["ctf/out"] = ctf.numpy()
    out["ctf/defocus_offsets"] = dfo.numpy()
    out["ctf/pixel_size_offsets"] = pxo.numpy()
    path = os.path.join(HERE, "preprocess_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__" and "--preprocess" in sys.argv:
    main_preprocess([a for a in sys.argv[1:] if a != "--preprocess"][0])
    sys.exit(0)

if __name__ == "__main__" and "--xcorr" in sys.argv:
    main_xcorr([a for a in sys.argv[1:] if a != "--xcorr"][0])
    sys.exit(0)

if __name__ == "__main__" and "--peaks" in sys.argv:
    main_peaks([a for a in sys.argv[1:] if a != "--peaks"][0])
    sys.exit(0)

if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
