"""CPU oracle for the search's pre-processing (TEST INFRASTRUCTURE ONLY).

Only ``tests/`` may import this module, as the checker of the device kernels
in ``leopard_em_gb300/csrc/preprocess.cu``; the product never imports it.

Restated in numpy float64:

* ``preprocess_image`` -- utils/image_processing.py:16-75: multiply by the
  cumulative filter, divide by the root of the total power (interior rfft
  columns counted twice), multiply by the root of the bandpass
  "dimensionality" (the same weighted count) and by the root of the
  image-to-box area ratio.  Pinned by ``tests/golden/preprocess_small.npz``
  (recorded from the reference's own function).
* ``whitening_filter`` -- the published construction of torch-fourier-filter's
  ``whitening_filter`` (called at config/correlation_filters.py:49-108; the
  package is not installed, parity unpinned): radial average of |F|^2 (or |F|)
  in ``num_bins`` nearest bins over [0, max_freq] cycles/pixel, inverted
  (square root for power), normalised to maximum 1, sampled by nearest bin on
  the output rfft grid.
* ``bandpass_filter`` -- torch-fourier-filter's ``bandpass_filter`` as used at
  correlation_filters.py:234-271: a band [low, high] cycles/pixel with
  raised-cosine edges of width ``falloff`` (hard when 0); parity unpinned.
* ``ctf_filter_stack`` -- ``oracle.ref_refine_template.ctf_filter_stack_full_args``
  (ctf_utils.py:19-116), whose wrapper logic is pinned by the same golden file.
"""

from __future__ import annotations

import numpy as np
import torch

from . import ref_refine_template as orr


def _radius(h: int, w: int) -> np.ndarray:
    ky = np.fft.fftfreq(h)[:, None]
    kx = np.fft.rfftfreq(w)[None, :]
    return np.sqrt(kx * kx + ky * ky)


def preprocess_image(image_rfft, filters, bandpass, full_image_shape, extracted_box_shape) -> np.ndarray:
    F = np.asarray(image_rfft, dtype=np.complex128) * np.asarray(filters, dtype=np.float64)
    sq = np.abs(F) ** 2
    ssum = sq.sum(axis=(-2, -1), keepdims=True) + sq[..., :, 1:-1].sum(axis=(-2, -1), keepdims=True)
    b = np.asarray(bandpass, dtype=np.float64)
    dim = b.sum() + b[:, 1:-1].sum()
    (ih, iw), (bh, bw) = full_image_shape, extracted_box_shape
    return F / np.sqrt(ssum) * np.sqrt(dim) * np.sqrt((ih * iw) / (bh * bw))


def whitening_filter(image_rfft, output_shape, num_bins=None, max_freq=0.5, do_power_spectrum=True) -> np.ndarray:
    F = np.asarray(image_rfft)
    H, wc = F.shape[-2:]
    W = 2 * (wc - 1)
    nb = num_bins or (max(H, W) // 2 + 1)
    fmax = 0.5 if max_freq is None else float(max_freq)
    idx = np.clip(np.rint(_radius(H, W) / fmax * (nb - 1)).astype(np.int64), 0, nb - 1)
    mag = np.abs(F.astype(np.complex128))
    val = mag**2 if do_power_spectrum else mag
    s = np.bincount(idx.ravel(), weights=val.ravel(), minlength=nb)
    c = np.bincount(idx.ravel(), minlength=nb).astype(np.float64)
    spec = s / np.maximum(c, 1.0)
    if do_power_spectrum:
        spec = np.sqrt(spec)
    f = np.where(spec > 0, 1.0 / np.where(spec > 0, spec, 1.0), 0.0)
    f = f / f.max()
    oh, ow = output_shape
    idx2 = np.clip(np.rint(_radius(oh, ow) / fmax * (nb - 1)).astype(np.int64), 0, nb - 1)
    return f[idx2]


def bandpass_filter(shape, low, high, falloff) -> np.ndarray:
    r = _radius(*shape)
    if falloff > 0:
        f = np.ones_like(r)
        f = np.where(r < low, 0.5 * (1 + np.cos(np.pi * np.clip((low - r) / falloff, 0, 1))), f)
        f = np.where(r > high, 0.5 * (1 + np.cos(np.pi * np.clip((r - high) / falloff, 0, 1))), f)
        return f
    return ((r >= low) & (r <= high)).astype(np.float64)


def ctf_filter_stack(template_size, defocus_u, defocus_v, defocus_offsets, pixel_size_offsets, **kw) -> np.ndarray:
    return orr.ctf_filter_stack_full_args((template_size, template_size), defocus_u, defocus_v,
                                          torch.as_tensor(defocus_offsets, dtype=torch.float32),
                                          torch.as_tensor(pixel_size_offsets, dtype=torch.float32), **kw).numpy()
