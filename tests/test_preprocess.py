"""Pre-processing: the oracle pinned to the reference's preprocess_image and
CTF-stack wrapper (golden vectors), the package's host (torch) path against
the oracle, and the device kernels (csrc/preprocess.cu, through the C ABI)
against the oracle.

Tolerances: spectra and filters within 1e-5 of their largest magnitude (FP32
data, FP64 sums on both sides); CTF within 2e-5 absolute (FP64 phase, FP32
output, |CTF| <= 1).
"""

import os

import numpy as np
import pytest
import torch

from leopard_em_gb300 import preprocess as pp
from oracle import ref_preprocess as orp

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "preprocess_small.npz"))
CTF_KW = dict(astigmatism_angle=25.0, voltage=300.0, spherical_aberration=2.7, amplitude_contrast_ratio=0.07,
              ctf_B_factor=60.0, phase_shift=0.0, pixel_size=1.06)


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def test_oracle_preprocess_image_matches_reference_golden():
    for case, shapes in (("single", ((96, 128), (96, 128))), ("stack", ((64, 64), (49, 49)))):
        got = orp.preprocess_image(GOLD[f"{case}/image_dft"], GOLD[f"{case}/filter"], GOLD[f"{case}/bandpass"],
                                   *shapes)
        assert _rel(got, GOLD[f"{case}/out"]) < 1e-5, case


def test_oracle_ctf_stack_matches_reference_wrapper():
    got = orp.ctf_filter_stack(32, 5200.0, 4950.0, GOLD["ctf/defocus_offsets"], GOLD["ctf/pixel_size_offsets"],
                               **CTF_KW)
    assert got.shape == (2, 3, 32, 17)
    assert np.abs(got - GOLD["ctf/out"]).max() < 1e-6


def _ctf_package(device):
    return pp.ctf_filter_stack(32, 5200.0, 4950.0, torch.tensor([-200.0, 0.0, 200.0]), torch.tensor([-0.02, 0.02]),
                               astigmatism_angle=25.0, voltage=300.0, spherical_aberration=2.7, amplitude_contrast=0.07,
                               phase_shift=0.0, pixel_size=1.06, b_factor=60.0, device=device)


def _image(h, w, seed):
    g = torch.Generator().manual_seed(seed)
    f = torch.fft.rfftn(torch.randn(h, w, generator=g) * (1.0 + torch.linspace(0, 1, w)))
    f[0, 0] = 0
    return f.to(torch.complex64)


def test_host_path_matches_oracle():
    assert np.abs(_ctf_package(None).numpy() - GOLD["ctf/out"]).max() < 2e-5
    img = _image(96, 128, 3)
    for nb, fmax, power in ((None, 0.5, True), (40, 0.4, False)):
        wf = pp.whitening_filter(img, (32, 32), num_bins=nb, max_freq=fmax, do_power_spectrum=power)
        ref = orp.whitening_filter(img.numpy(), (32, 32), nb, fmax, power)
        assert _rel(wf.numpy(), ref) < 1e-5
    bp = pp.bandpass_filter((96, 128), 0.05, 0.3, 0.05)
    assert np.abs(bp.numpy() - orp.bandpass_filter((96, 128), 0.05, 0.3, 0.05)).max() < 1e-6
    out = pp.preprocess_image(torch.from_numpy(GOLD["single/image_dft"]), torch.from_numpy(GOLD["single/filter"]),
                              torch.from_numpy(GOLD["single/bandpass"]), (96, 128), (96, 128))
    assert _rel(out.numpy(), GOLD["single/out"]) < 1e-5


@pytest.mark.gpu
def test_device_kernels_match_oracle():
    dev = torch.device("cuda:0")
    ctf = _ctf_package(dev)
    assert ctf.is_cuda and np.abs(ctf.cpu().numpy() - GOLD["ctf/out"]).max() < 2e-5
    for h, w in ((96, 128), (256, 288), (4096, 4096)):  # 256 x 288 has exact nearest-bin ties
        img = _image(h, w, 4)
        for out_shape, nb, fmax, power in (((32, 32), None, 0.5, True), ((h, w), 40, 0.4, False),
                                           ((384, 384), None, 0.5, True)):
            wf = pp.whitening_filter(img.to(dev), out_shape, num_bins=nb, max_freq=fmax, do_power_spectrum=power)
            ref = orp.whitening_filter(img.numpy(), out_shape, nb, fmax, power)
            assert wf.is_cuda and wf.shape == ref.shape
            assert _rel(wf.cpu().numpy(), ref) < 1e-5, (h, w, out_shape, nb)
    for lo, hi, fo in ((0.05, 0.3, 0.05), (0.0, 0.25, 0.0)):
        bp = pp.bandpass_filter((96, 128), lo, hi, fo, device=dev)
        assert np.abs(bp.cpu().numpy() - orp.bandpass_filter((96, 128), lo, hi, fo)).max() < 1e-6
    for case, shapes in (("single", ((96, 128), (96, 128))), ("stack", ((64, 64), (49, 49)))):
        out = pp.preprocess_image(torch.from_numpy(GOLD[f"{case}/image_dft"]).to(dev),
                                  torch.from_numpy(GOLD[f"{case}/filter"]).to(dev),
                                  torch.from_numpy(GOLD[f"{case}/bandpass"]).to(dev), *shapes)
        assert out.is_cuda and _rel(out.cpu().numpy(), GOLD[f"{case}/out"]) < 1e-5, case


@pytest.mark.gpu
def test_manager_inputs_on_device_match_host():
    """make_backend_core_function_kwargs with the device kernels equals the host path."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.managers import BandpassFilterConfig, PreprocessingFilters, calculate_ctf_filter_stack
    from leopard_em_gb300.managers import OpticsGroup

    img = torch.randn(256, 288, generator=torch.Generator().manual_seed(2))
    vol, _ = sy.blob_volume(32, 40, 1.5, 10.0, 0)
    pf = PreprocessingFilters(bandpass_filter=BandpassFilterConfig(enabled=True, low_freq_cutoff=0.02,
                                                                   high_freq_cutoff=0.4, falloff=0.02))
    og = OpticsGroup(label="x", pixel_size=1.0, voltage=300.0, defocus_u=10000.0, defocus_v=9800.0,
                     astigmatism_angle=30.0, ctf_B_factor=20.0)
    out = {}
    for dev in (torch.device("cpu"), torch.device("cuda:0")):
        f = torch.fft.rfftn(img.to(dev))
        f[0, 0] = 0
        bp = pf.bandpass_filter.calculate_bandpass_filter(f.shape, device=dev)
        cum = pf.get_combined_filter(f, tuple(f.shape))
        out[dev.type] = {
            "image": pp.preprocess_image(f, cum, bp, (256, 288), (256, 288)),
            "template_filter": pf.get_combined_filter(f, (32, 17)),
            "ctf": calculate_ctf_filter_stack((32, 32), og, torch.tensor([-100.0, 0.0, 100.0]), torch.tensor([0.0]),
                                              device=dev),
            "template": pp.volume_to_rfft_fourier_slice(vol.to(dev)),
        }
    for k in out["cpu"]:
        a, b = out["cpu"][k], out["cuda"][k].cpu()
        assert out["cuda"][k].is_cuda and a.shape == b.shape, k
        assert (a - b).abs().max().item() <= 1e-4 * max(1.0, a.abs().max().item()), k
