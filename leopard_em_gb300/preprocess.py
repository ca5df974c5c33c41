"""Preparation of the search inputs (torch, once per micrograph, on the
device of the tensors passed in: the GPU when the manager is given one).

These mirror what ``MatchTemplateManager.make_backend_core_function_kwargs``
does before calling the backend (match_template_manager.py:140-218):
  * ``volume_to_rfft_fourier_slice``  utils/image_processing.py:179-202
  * ``preprocess_image``              utils/image_processing.py:16-75
  * ``ctf_2d`` / ``ctf_filter_stack`` utils/ctf_utils.py:19-116, with the
    published CTF formula (the reference calls torch-ctf's calculate_ctf_2d)
  * ``get_cs_range``                  utils/search_utils.py:6-29
  * ``whitening_filter``              a radially averaged 1/sqrt(power) filter,
    the published construction of torch-fourier-filter's whitening_filter.
They are not part of the timed search.  Every function works on the device
of its input tensors: on a CUDA device the CTF stack, the whitening and
bandpass filters and the filter-and-normalise step run as this package's
kernels (``csrc/preprocess.cu``); on the CPU they run as torch operations.
The image and template rffts are torch.fft on either device.
"""

from __future__ import annotations

import math

import torch


def _on_cuda(device) -> bool:
    return device is not None and torch.device(device).type == "cuda"


def _native():
    from . import _native as nat

    return nat


def volume_to_rfft_fourier_slice(volume: torch.Tensor) -> torch.Tensor:
    """fftshift -> rfftn -> fftshift over the first two axes."""
    if volume.dim() != 3:
        raise ValueError("volume must be 3D")
    v = torch.fft.fftshift(volume, dim=(0, 1, 2))
    v = torch.fft.rfftn(v, dim=(0, 1, 2))
    return torch.fft.fftshift(v, dim=(0, 1))


def preprocess_image(image_rfft, cumulative_fourier_filters, bandpass_filter, full_image_shape, extracted_box_shape):
    """Filter, normalise to unit power, scale by sqrt(dimensionality) and box area."""
    if image_rfft.is_cuda:
        return _preprocess_image_native(image_rfft, cumulative_fourier_filters, bandpass_filter, full_image_shape,
                                        extracted_box_shape)
    image_rfft = image_rfft * cumulative_fourier_filters
    sq = torch.abs(image_rfft) ** 2
    ssum = torch.sum(sq, dim=(-2, -1), keepdim=True)
    ssum = ssum + torch.sum(sq[..., :, 1:-1], dim=(-2, -1), keepdim=True)
    image_rfft = image_rfft / torch.sqrt(ssum)
    dimensionality = bandpass_filter.sum() + bandpass_filter[:, 1:-1].sum()
    image_rfft = image_rfft * dimensionality**0.5
    img_h, img_w = full_image_shape
    box_h, box_w = extracted_box_shape
    return image_rfft * ((img_h * img_w) / (box_h * box_w)) ** 0.5


def _preprocess_image_native(image_rfft, filters, bandpass, full_image_shape, extracted_box_shape):
    import ctypes

    nat = _native()
    dev = image_rfft.device
    H, wc = image_rfft.shape[-2:]
    n = 1 if image_rfft.dim() == 2 else int(image_rfft.shape[0])
    F = image_rfft.to(torch.complex64).reshape(n, H, wc).contiguous()
    f = filters.to(dev, torch.float32)
    if f.dim() == 3 and f.shape[0] == n and n > 1:
        f = f.contiguous()
        stride = H * wc
    else:
        f = f.reshape(H, wc).contiguous()
        stride = 0
    bp = bandpass.to(dev, torch.float32).reshape(H, wc).contiguous()
    out = torch.empty_like(F)
    scratch = torch.empty(n + 1, dtype=torch.float64, device=dev)
    (ih, iw), (bh, bw) = full_image_shape, extracted_box_shape
    with torch.cuda.device(dev):
        s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        nat.check(nat.lib().lgb_preprocess_image(n, H, 2 * (wc - 1), F.data_ptr(), f.data_ptr(), stride,
                                                 bp.data_ptr(), float(ih * iw) / float(bh * bw),
                                                 scratch.data_ptr(), out.data_ptr(), s), "preprocess_image")
    return out.reshape(image_rfft.shape)


def rfft_freq_grid(shape: tuple[int, int], pixel_size: float = 1.0, device=None):
    """(ky, kx) spatial frequencies (1/Angstrom) of an unshifted rfft grid."""
    h, w = shape
    ky = torch.fft.fftfreq(h, dtype=torch.float64, device=device)[:, None] / pixel_size
    kx = torch.fft.rfftfreq(w, dtype=torch.float64, device=device)[None, :] / pixel_size
    return ky.expand(h, w // 2 + 1), kx.expand(h, w // 2 + 1)


def electron_wavelength(voltage_kv: float) -> float:
    """Relativistic electron wavelength in Angstrom."""
    v = voltage_kv * 1e3
    h, m0, e, c = 6.62607015e-34, 9.1093837015e-31, 1.602176634e-19, 299792458.0
    return h / math.sqrt(2 * m0 * e * v * (1 + e * v / (2 * m0 * c * c))) * 1e10


def ctf_2d(
    shape: tuple[int, int],
    defocus: float,
    astigmatism: float = 0.0,
    astigmatism_angle: float = 0.0,
    voltage: float = 300.0,
    spherical_aberration: float = 2.7,
    amplitude_contrast: float = 0.07,
    phase_shift: float = 0.0,
    pixel_size: float = 1.0,
    b_factor: float = 0.0,
    device=None,
) -> torch.Tensor:
    """CTF on an unshifted rfft grid: -sin(chi), defocus/astigmatism in Angstrom.

    chi = pi*lambda*k^2*df(theta) - pi/2*Cs*lambda^3*k^4 + phase + asin(A)-term,
    with df(theta) = defocus + astigmatism*cos(2(theta - angle)), written in the
    sign convention -sin(-pi lambda df k^2 + pi/2 Cs lambda^3 k^4 - phi - atan(A/sqrt(1-A^2))),
    and an optional B-factor envelope exp(-B k^2 / 4).
    """
    ky, kx = rfft_freq_grid(shape, pixel_size, device)
    k2 = kx**2 + ky**2
    lam = electron_wavelength(voltage)
    cs = spherical_aberration * 1e7
    ang = torch.atan2(ky, kx)
    df = defocus + astigmatism * torch.cos(2 * (ang - math.radians(astigmatism_angle)))
    k5 = math.atan(amplitude_contrast / math.sqrt(1 - amplitude_contrast**2))
    chi = -math.pi * lam * k2 * df + 0.5 * math.pi * cs * lam**3 * k2**2 - math.radians(phase_shift) - k5
    out = -torch.sin(chi)
    if b_factor:
        out = out * torch.exp(-b_factor * k2 / 4)
    return out.to(torch.float32)


def get_cs_range(pixel_size: float, pixel_size_offsets: torch.Tensor, cs: float = 2.7) -> torch.Tensor:
    """Cs values emulating relative pixel-size changes (search_utils.py:6-29)."""
    return cs / torch.pow((pixel_size + pixel_size_offsets) / pixel_size, 4)


def ctf_filter_stack(
    template_size: int,
    defocus_u: float,
    defocus_v: float,
    defocus_offsets: torch.Tensor,
    pixel_size_offsets: torch.Tensor,
    astigmatism_angle: float = 0.0,
    voltage: float = 300.0,
    spherical_aberration: float = 2.7,
    amplitude_contrast: float = 0.07,
    phase_shift: float = 0.0,
    pixel_size: float = 1.0,
    b_factor: float = 0.0,
    device=None,
) -> torch.Tensor:
    """(num_pixel_sizes, num_defocus, d, d//2+1) stack as ctf_utils.py:19-116."""
    if _on_cuda(device):
        return _ctf_filter_stack_native(template_size, defocus_u, defocus_v, defocus_offsets, pixel_size_offsets,
                                        astigmatism_angle, voltage, spherical_aberration, amplitude_contrast,
                                        phase_shift, pixel_size, b_factor, torch.device(device))
    mean_df = (defocus_u + defocus_v) / 2
    astig = abs(defocus_u - defocus_v) / 2
    cs_values = get_cs_range(pixel_size, pixel_size_offsets, spherical_aberration)
    stack = []
    for cs in cs_values.tolist():
        stack.append(
            torch.stack(
                [
                    ctf_2d((template_size, template_size), mean_df + float(o), astig, astigmatism_angle, voltage, cs,
                           amplitude_contrast, phase_shift, pixel_size, b_factor, device)
                    for o in defocus_offsets.tolist()
                ]
            )
        )
    return torch.stack(stack)


def _ctf_filter_stack_native(d, du, dv, dfo, pxo, ang, voltage, cs, amp, phase, px, b, dev):
    import ctypes

    nat = _native()
    dfo = torch.as_tensor(dfo, dtype=torch.float32).reshape(-1).to(dev).contiguous()
    pxo = torch.as_tensor(pxo, dtype=torch.float32).reshape(-1).to(dev).contiguous()
    out = torch.empty((pxo.numel(), dfo.numel(), d, d // 2 + 1), dtype=torch.float32, device=dev)
    prm = nat.CtfParams(voltage_kv=float(voltage), spherical_aberration_mm=float(cs),
                        amplitude_contrast=float(amp), b_factor=float(b), phase_shift_deg=float(phase),
                        pixel_size=float(px))
    with torch.cuda.device(dev):
        s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        nat.check(nat.lib().lgb_ctf_filter_stack(int(d), float(du), float(dv), float(ang), ctypes.byref(prm),
                                                 dfo.data_ptr(), dfo.numel(), pxo.data_ptr(), pxo.numel(),
                                                 out.data_ptr(), s), "ctf_filter_stack")
    return out


def _whitening_filter_native(image_rfft, output_shape, nb, fmax, power):
    import ctypes

    nat = _native()
    dev = image_rfft.device
    H, wc = image_rfft.shape[-2:]
    n = 1 if image_rfft.dim() == 2 else int(image_rfft.shape[0])
    F = image_rfft.to(torch.complex64).reshape(n, H, wc).contiguous()
    bsum = torch.empty((n, nb), dtype=torch.float64, device=dev)
    bcnt = torch.empty((n, nb), dtype=torch.float64, device=dev)
    oh, ow = output_shape
    out = torch.empty((n, oh, ow // 2 + 1), dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        L = nat.lib()
        nat.check(L.lgb_radial_spectrum(n, H, 2 * (wc - 1), F.data_ptr(), nb, float(fmax), int(power),
                                        bsum.data_ptr(), bcnt.data_ptr(), s), "radial_spectrum")
        nat.check(L.lgb_whitening_filter(n, nb, float(fmax), int(power), bsum.data_ptr(), bcnt.data_ptr(), oh, ow,
                                         out.data_ptr(), s), "whitening_filter")
    return out[0] if image_rfft.dim() == 2 else out


def whitening_filter(image_rfft: torch.Tensor, output_shape: tuple[int, int], num_bins: int | None = None,
                     max_freq: float | None = 0.5, do_power_spectrum: bool = True):
    """Whitening filter of ``image_rfft`` sampled on the rfft grid of real shape
    ``output_shape``, normalised to max 1 (the published construction of
    torch-fourier-filter's whitening_filter, called at
    config/correlation_filters.py:97-108): the radially averaged power
    (|F|^2, or |F| when ``do_power_spectrum`` is False) in ``num_bins`` bins
    over [0, max_freq] cycles/pixel, inverted (square root for power), and
    sampled at each output frequency by its nearest bin; frequencies beyond
    ``max_freq`` take the last bin's value."""
    H = image_rfft.shape[-2]
    W = 2 * (image_rfft.shape[-1] - 1)
    dev = image_rfft.device
    fmax = 0.5 if max_freq is None else float(max_freq)
    if fmax <= 0:
        raise ValueError("max_freq must be > 0")
    nb = num_bins or int(max(H, W) // 2 + 1)
    if image_rfft.is_cuda:
        return _whitening_filter_native(image_rfft, tuple(output_shape), nb, fmax, do_power_spectrum)
    ky, kx = rfft_freq_grid((H, W), device=dev)
    r = torch.sqrt(kx**2 + ky**2)
    idx = torch.clamp((r / fmax * (nb - 1)).round().long(), 0, nb - 1)
    mag = image_rfft.abs().double()
    val = mag**2 if do_power_spectrum else mag
    power = torch.zeros(nb, dtype=torch.float64, device=dev).index_add_(0, idx.flatten(), val.flatten())
    count = torch.zeros(nb, dtype=torch.float64, device=dev).index_add_(
        0, idx.flatten(), torch.ones(idx.numel(), dtype=torch.float64, device=dev))
    spec = power / count.clamp_min(1)
    if do_power_spectrum:
        spec = torch.sqrt(spec)
    filt1d = torch.where(spec > 0, 1.0 / spec, torch.zeros_like(spec))
    filt1d = filt1d / filt1d.max()
    ky2, kx2 = rfft_freq_grid(output_shape, device=dev)
    r2 = torch.sqrt(kx2**2 + ky2**2)
    idx2 = torch.clamp((r2 / fmax * (nb - 1)).round().long(), 0, nb - 1)
    return filt1d[idx2].to(torch.float32)


def bandpass_filter(shape: tuple[int, int], low: float, high: float, falloff: float, device=None) -> torch.Tensor:
    """Band [low, high] cycles/pixel on the rfft grid of real ``shape`` with
    raised-cosine edges of width ``falloff`` (a hard band when falloff = 0);
    the published form of torch-fourier-filter's bandpass_filter
    (config/correlation_filters.py:234-271)."""
    if _on_cuda(device):
        import ctypes

        nat = _native()
        dev = torch.device(device)
        h, w = shape
        out = torch.empty((h, w // 2 + 1), dtype=torch.float32, device=dev)
        with torch.cuda.device(dev):
            s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            nat.check(nat.lib().lgb_bandpass_filter(int(h), int(w), float(low), float(high), float(falloff),
                                                    out.data_ptr(), s), "bandpass_filter")
        return out
    ky, kx = rfft_freq_grid(shape, device=device)
    r = torch.sqrt(kx**2 + ky**2)
    f = torch.ones_like(r)
    if falloff > 0:
        f = torch.where(r < low, 0.5 * (1 + torch.cos(math.pi * torch.clamp((low - r) / falloff, 0, 1))), f)
        f = torch.where(r > high, 0.5 * (1 + torch.cos(math.pi * torch.clamp((r - high) / falloff, 0, 1))), f)
    else:
        f = ((r >= low) & (r <= high)).to(r.dtype)
    return f.to(torch.float32)


def radial_curve_filter(shape: tuple[int, int], frequencies, amplitudes, device=None) -> torch.Tensor:
    """A 1-D amplitude curve (cycles/pixel -> amplitude) placed radially on the
    rfft grid of real ``shape`` by linear interpolation, 1 outside the curve's
    range (curve_1dim_to_ndim with fill 1, config/correlation_filters.py:290-336)."""
    f = torch.as_tensor(frequencies, dtype=torch.float64, device=device)
    a = torch.as_tensor(amplitudes, dtype=torch.float64, device=device)
    if f.numel() != a.numel() or f.numel() < 1:
        raise ValueError("frequencies and amplitudes must be non-empty and of equal length")
    order = torch.argsort(f)
    f, a = f[order], a[order]
    ky, kx = rfft_freq_grid(shape, device=device)
    r = torch.sqrt(kx**2 + ky**2)
    j = torch.searchsorted(f, r.contiguous()).clamp(1, max(1, f.numel() - 1))
    if f.numel() == 1:
        out = torch.where(r == f[0], a[0], torch.ones_like(r))
    else:
        f0, f1, a0, a1 = f[j - 1], f[j], a[j - 1], a[j]
        t = ((r - f0) / (f1 - f0).clamp_min(1e-30)).clamp(0, 1)
        out = a0 + t * (a1 - a0)
        out = torch.where((r < f[0]) | (r > f[-1]), torch.ones_like(r), out)
    return out.to(torch.float32)
