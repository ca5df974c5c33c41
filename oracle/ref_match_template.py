"""CPU oracle for the 2DTM whole-orientation search (TEST INFRASTRUCTURE ONLY).

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  The product path (``leopard_em_gb300``) never imports it and fails loudly
when its CUDA library is missing.

It restates, on the CPU with ``torch.fft`` (pocketfft), the exact operation
sequence of Leopard-EM's search backend:

* ``euler_to_rotmat_zyz``  -- roma ``euler_to_rotmat("ZYZ", degrees=True)``
  (third-party, unpinned version; published convention: intrinsic Z-Y-Z,
  R = Rz(phi) @ Ry(theta) @ Rz(psi)).  Called at
  ``backend/core_match_template.py:506-508``.
* ``extract_central_slices_rfft_3d`` -- torch-fourier-slice >= 0.4.0
  (third-party, not vendored).  Published algorithm: a central-slice grid of
  (z=0, y=fftshift(fftfreq(d)), x=rfftfreq(d)) frequencies, rotated by the
  zyx-flipped rotation matrix, points with x<0 mirrored to the Friedel mate and
  conjugated, frequencies mapped to array indices of the fftshifted rfft volume
  (``f*d + d//2`` on z/y, ``f*d`` on x), trilinear interpolation, zero outside
  the volume.  Called at ``backend/cross_correlation.py:76-79``.
* ``normalize_template_projection`` -- ``backend/utils.py:106-188``.
* ``cross_correlate_streamed`` -- ``backend/cross_correlation.py:13-154``.
* ``cross_correlate_batched_cpu`` -- ``backend/cross_correlation.py:287-369``.
* ``iteration_statistics_update`` -- ``backend/utils.py:191-255``.
* ``decode_global_search_index`` / ``scale_mip`` --
  ``backend/process_results.py:67-183``.
* ``core_match_template_cpu`` -- the orientation loop of
  ``backend/core_match_template.py:274-277, 458-466, 492-550`` and the epilogue
  ``:329-363``, with the same argument names and return keys.

Parity pin: ``tests/golden/make_golden.py`` imports the reference's own
``cross_correlation.py``, ``utils.py`` and ``process_results.py`` from the
reference source tree (with roma / torch_fourier_slice replaced by the two
restatements above, because those packages are not installed) and records
input/output vectors under ``tests/golden/``; ``tests/test_oracle_golden.py``
checks this module against them.  The two third-party restatements themselves
are pinned only by self-consistency checks (projection-slice theorem on an
analytic Gaussian-blob volume, planted-particle recovery), because the
third-party packages cannot be installed here.
"""

from __future__ import annotations

import math

import numpy as np
import torch

# ---------------------------------------------------------------------------
# Third-party restatements
# ---------------------------------------------------------------------------


def euler_to_rotmat_zyz(euler_deg: torch.Tensor, dtype=torch.float32) -> torch.Tensor:
    """Intrinsic ZYZ Euler angles in degrees -> rotation matrices (..., 3, 3).

    R = Rz(phi) @ Ry(theta) @ Rz(psi), the convention of
    ``roma.euler_to_rotmat("ZYZ", angles, degrees=True)``.
    """
    a = torch.deg2rad(euler_deg.to(dtype))
    phi, theta, psi = a[..., 0], a[..., 1], a[..., 2]

    def rz(t):
        c, s = torch.cos(t), torch.sin(t)
        z, o = torch.zeros_like(t), torch.ones_like(t)
        return torch.stack(
            [torch.stack([c, -s, z], -1), torch.stack([s, c, z], -1), torch.stack([z, z, o], -1)], -2
        )

    def ry(t):
        c, s = torch.cos(t), torch.sin(t)
        z, o = torch.zeros_like(t), torch.ones_like(t)
        return torch.stack(
            [torch.stack([c, z, s], -1), torch.stack([z, o, z], -1), torch.stack([-s, z, c], -1)], -2
        )

    return rz(phi) @ ry(theta) @ rz(psi)


def _trilinear_zero_outside(volume: torch.Tensor, coords: torch.Tensor) -> torch.Tensor:
    """Trilinear sample of a (d0, d1, d2) complex volume at (..., 3) zyx index coords.

    Points outside [0, n-1] on any axis give 0 (grid_sample 'border' padding with
    align_corners=True followed by explicit zeroing of outside samples).
    """
    shape = volume.shape
    flat = coords.reshape(-1, 3)
    dims = torch.tensor(shape, dtype=flat.dtype, device=flat.device)
    inside = ((flat >= 0) & (flat <= dims - 1)).all(dim=-1)
    c = torch.minimum(torch.clamp(flat, min=0.0), dims - 1)
    i0 = torch.floor(c).long()
    t = c - i0.to(c.dtype)
    i1 = torch.minimum(i0 + 1, (dims - 1).long())
    out = torch.zeros(flat.shape[0], dtype=volume.dtype, device=volume.device)
    for dz in (0, 1):
        iz = i1[:, 0] if dz else i0[:, 0]
        wz = t[:, 0] if dz else 1 - t[:, 0]
        for dy in (0, 1):
            iy = i1[:, 1] if dy else i0[:, 1]
            wy = t[:, 1] if dy else 1 - t[:, 1]
            for dx in (0, 1):
                ix = i1[:, 2] if dx else i0[:, 2]
                wx = t[:, 2] if dx else 1 - t[:, 2]
                w = (wz * wy * wx).to(volume.real.dtype)
                out = out + volume[iz, iy, ix] * w
    out = torch.where(inside, out, torch.zeros_like(out))
    return out.reshape(coords.shape[:-1])


def extract_central_slices_rfft_3d(
    volume_rfft: torch.Tensor, rotation_matrices: torch.Tensor
) -> torch.Tensor:
    """Central slices (..., d, d//2+1) of an fftshifted rfft volume (d, d, d//2+1).

    Output rows are fftshifted (DC at row d//2), as in torch-fourier-slice.
    """
    d = volume_rfft.shape[0]
    rdtype = volume_rfft.real.dtype
    dev = volume_rfft.device
    fy = torch.fft.fftshift(torch.fft.fftfreq(d, dtype=rdtype, device=dev))
    fx = torch.fft.rfftfreq(d, dtype=rdtype, device=dev)
    gy, gx = torch.meshgrid(fy, fx, indexing="ij")
    zyx = torch.stack([torch.zeros_like(gy), gy, gx], dim=-1)  # (d, wc, 3)
    r_zyx = torch.flip(rotation_matrices.to(dev, rdtype), dims=(-2, -1))
    rot = torch.einsum("...ij,hwj->...hwi", r_zyx, zyx)
    conj = rot[..., 2] < 0
    rot = torch.where(conj[..., None], -rot, rot)
    dc = torch.tensor([d // 2, d // 2, 0], dtype=rdtype, device=dev)
    coords = rot * d + dc
    samples = _trilinear_zero_outside(volume_rfft, coords)
    return torch.where(conj, samples.conj(), samples)


# ---------------------------------------------------------------------------
# Leopard-EM backend restatement
# ---------------------------------------------------------------------------


def normalize_template_projection(projections, small_shape, large_shape):
    """Edge-mean subtraction and padded-variance normalisation (utils.py:106-188)."""
    top = projections[..., 0, :]
    bottom = projections[..., -1, :]
    left = projections[..., 1:-1, 0]
    right = projections[..., 1:-1, -1]
    edge = torch.concatenate([top, bottom, left, right], dim=-1)
    projections = projections - edge.mean(dim=-1)[..., None, None]
    large_size_sqrt = (large_shape[0] * large_shape[1]) ** 0.5
    relative_size = (small_shape[0] * small_shape[1]) / (large_shape[0] * large_shape[1])
    mean = torch.mean(projections, dim=(-2, -1), keepdim=True) * relative_size
    mean = mean * relative_size  # the reference scales by relative_size twice
    variance = torch.sum((projections - mean) ** 2, dim=(-2, -1), keepdim=True)
    variance = variance + (large_shape[0] - small_shape[0]) * (large_shape[1] - small_shape[1]) * mean**2
    return (projections * large_size_sqrt) / torch.sqrt(variance.clamp_min(1e-8))


def prepare_fourier_slices(template_dft, rotation_matrices):
    """Slices -> ifftshift rows -> DC=0 -> contrast flip (cross_correlation.py:76-92)."""
    fs = extract_central_slices_rfft_3d(template_dft, rotation_matrices)
    fs = torch.fft.ifftshift(fs, dim=(-2,))
    fs[..., 0, 0] = 0 + 0j
    fs = fs * -1
    return fs


def cross_correlate_streamed(image_dft, template_dft, rotation_matrices, projective_filters):
    """One CC at a time, as ``do_streamed_orientation_cross_correlate`` (:13-154)."""
    proj_shape = (template_dft.shape[1], template_dft.shape[2] * 2 - 2)
    img_shape = (image_dft.shape[0], image_dft.shape[1] * 2 - 2)
    n_o = rotation_matrices.shape[0]
    n_cs, n_df = projective_filters.shape[0], projective_filters.shape[1]
    out = torch.empty((n_cs, n_df, n_o, *img_shape), dtype=image_dft.real.dtype, device=image_dft.device)
    fs_all = prepare_fourier_slices(template_dft, rotation_matrices)
    for i in range(n_o):
        for j in range(n_df):
            for k in range(n_cs):
                fsf = fs_all[i] * projective_filters[k, j]
                proj = torch.fft.irfft2(fsf)
                proj = torch.fft.ifftshift(proj, dim=(-2, -1))
                proj = normalize_template_projection(proj, proj_shape, img_shape)
                tmp = torch.fft.rfft(proj, n=img_shape[1], dim=-1)
                pdft = torch.fft.fft(tmp, n=img_shape[0], dim=-2)
                pdft[0, 0] = 0 + 0j
                pdft = image_dft * pdft.conj()
                out[k, j, i] = torch.fft.irfft2(pdft, s=img_shape)
    return out


def cross_correlate_batched_cpu(image_dft, template_dft, rotation_matrices, projective_filters):
    """Batched form, as ``do_batched_orientation_cross_correlate_cpu`` (:287-369)."""
    proj_shape = (template_dft.shape[1], template_dft.shape[2] * 2 - 2)
    img_shape = (image_dft.shape[0], image_dft.shape[1] * 2 - 2)
    fs = prepare_fourier_slices(template_dft, rotation_matrices)
    fs = fs[None, None, ...] * projective_filters[:, :, None, ...]
    proj = torch.fft.irfftn(fs, dim=(-2, -1))
    proj = torch.fft.ifftshift(proj, dim=(-2, -1))
    proj = normalize_template_projection(proj, proj_shape, img_shape)
    pdft = torch.fft.rfftn(proj, dim=(-2, -1), s=img_shape)
    pdft[..., 0, 0] = 0 + 0j
    pdft = image_dft[None, None, None, ...] * pdft.conj()
    return torch.fft.irfftn(pdft, dim=(-2, -1))


def iteration_statistics_update(
    cross_correlation, current_indexes, mip, best_global_index, correlation_sum,
    correlation_squared_sum, img_h, img_w, second_best=None,
):
    """Per-batch MIP / argmax / sum / sum-of-squares update (utils.py:191-255).

    ``second_best`` (optional extra map) tracks the runner-up value per pixel so
    that parity tests can tell ties from genuine argmax disagreements.
    """
    cc = cross_correlation.reshape(-1, img_h, img_w)
    max_values, max_indices = torch.max(cc, dim=0)
    if second_best is not None:
        if cc.shape[0] > 1:
            top2 = torch.topk(cc, 2, dim=0).values
            batch_second = top2[1]
        else:
            batch_second = torch.full_like(max_values, -float("inf"))
        new_second = torch.maximum(torch.minimum(max_values, mip), torch.maximum(second_best, batch_second))
        second_best.copy_(new_second)
    update = max_values > mip
    torch.where(update, max_values, mip, out=mip)
    torch.where(update, current_indexes[max_indices], best_global_index, out=best_global_index)
    correlation_sum += cc.to(correlation_sum.dtype).sum(dim=0)
    correlation_squared_sum += (cc.to(correlation_squared_sum.dtype) ** 2).sum(dim=0)


def decode_global_search_index(global_indices, pixel_values, defocus_values, euler_angles):
    """Global index -> (phi, theta, psi, defocus) (process_results.py:67-95)."""
    n_df = defocus_values.shape[0]
    n_o = euler_angles.shape[0]
    rem = global_indices.long() % (n_df * n_o)
    df_idx = rem // n_o
    o_idx = rem % n_o
    return euler_angles[o_idx, 0], euler_angles[o_idx, 1], euler_angles[o_idx, 2], defocus_values[df_idx]


def scale_mip(mip, correlation_sum, correlation_squared_sum, total_correlation_positions):
    """Mean, std ("variance" key) and z-score map (process_results.py:98-183)."""
    mean = correlation_sum / total_correlation_positions
    var = correlation_squared_sum / total_correlation_positions
    var = var - mean**2
    std = torch.sqrt(torch.clamp(var, min=0))
    scaled = mip - mean
    scaled = torch.where(std != 0, scaled / std, torch.zeros_like(scaled))
    return mip, scaled, mean, std


def core_match_template_cpu(
    image_dft, template_dft, ctf_filters, whitening_filter_template, defocus_values,
    pixel_values, euler_angles, orientation_batch_size=1, backend="streamed",
    stat_dtype=torch.float32, track_second_best=False, compute_dtype=torch.float32, device=None,
):
    """CPU restatement of ``core_match_template`` (core_match_template.py:146-363).

    ``stat_dtype`` float32 reproduces the reference's statistics accumulation
    (``DEFAULT_STATISTIC_DTYPE``, :31); float64 gives the FP64 oracle.
    ``compute_dtype`` float64 runs the whole correlation in double precision.
    ``device`` runs the same torch operations elsewhere (a CUDA device makes an
    FP64 oracle of many orientations affordable); results come back on the CPU.
    The last partial orientation batch gets exactly as many global indices as it
    has orientations (the reference always generates a full batch, :513-520).
    """
    dev = torch.device(device) if device is not None else torch.device("cpu")
    cdt = torch.complex128 if compute_dtype == torch.float64 else torch.complex64
    image_dft = image_dft.to(dev, cdt)
    template_dft = template_dft.to(dev, cdt)
    pf = (ctf_filters.to(dev) * whitening_filter_template.to(dev)[None, None, ...]).to(compute_dtype)
    euler_angles = euler_angles.to(torch.float32)
    n_o, n_df, n_cs = euler_angles.shape[0], defocus_values.shape[0], pixel_values.shape[0]
    total = n_o * n_df * n_cs
    img_shape = (image_dft.shape[0], image_dft.shape[1] * 2 - 2)
    incr = torch.tensor(
        [df * n_o + cs * n_df * n_o for cs in range(n_cs) for df in range(n_df)], dtype=torch.int64, device=dev
    )
    mip = torch.full(img_shape, -float("inf"), dtype=compute_dtype, device=dev)
    best = torch.full(img_shape, -1, dtype=torch.int64, device=dev)
    s1 = torch.zeros(img_shape, dtype=stat_dtype, device=dev)
    s2 = torch.zeros(img_shape, dtype=stat_dtype, device=dev)
    second = torch.full(img_shape, -float("inf"), dtype=compute_dtype, device=dev) if track_second_best else None
    B = orientation_batch_size
    for i in range(0, n_o, B):
        eb = euler_angles[i : i + B]
        rot = euler_to_rotmat_zyz(eb, dtype=compute_dtype).to(dev)
        idx = torch.arange(i, i + eb.shape[0], dtype=torch.int64, device=dev)
        bsi = (idx + incr[:, None]).flatten()
        if backend == "batched":
            cc = cross_correlate_batched_cpu(image_dft, template_dft, rot, pf)
        else:
            cc = cross_correlate_streamed(image_dft, template_dft, rot, pf)
        iteration_statistics_update(cc, bsi, mip, best, s1, s2, img_shape[0], img_shape[1], second)
    best, mip, s1, s2 = best.cpu(), mip.cpu(), s1.cpu(), s2.cpu()
    second = second.cpu() if second is not None else None
    phi, theta, psi, dfv = decode_global_search_index(best, pixel_values, defocus_values, euler_angles)
    mip, scaled, mean, std = scale_mip(mip, s1, s2, total)
    out = {
        "mip": mip,
        "scaled_mip": scaled,
        "best_phi": phi,
        "best_theta": theta,
        "best_psi": psi,
        "best_defocus": dfv,
        "correlation_mean": mean,
        "correlation_variance": std,
        "total_projections": total,
        "total_orientations": n_o,
        "total_defocus": n_df,
        "best_global_index": best,
    }
    if track_second_best:
        out["second_best"] = second
    return out


# ---------------------------------------------------------------------------
# Helpers the tests use to build inputs the same way the reference does
# ---------------------------------------------------------------------------


def volume_to_rfft_fourier_slice(volume: torch.Tensor) -> torch.Tensor:
    """fftshift -> rfftn -> fftshift(0, 1) (utils/image_processing.py:179-202)."""
    v = torch.fft.fftshift(volume, dim=(0, 1, 2))
    v = torch.fft.rfftn(v, dim=(0, 1, 2))
    return torch.fft.fftshift(v, dim=(0, 1))


def analytic_blob_projection(centres_xyz, sigma, rotation, size):
    """Line-integral projection of isotropic Gaussian blobs, for the
    projection-slice self-check.  Blob c projects to (R^T c)_xy, centred at
    pixel size//2.  Returns a (size, size) float64 array indexed [y, x]."""
    r = np.asarray(rotation, dtype=np.float64)
    p = np.asarray(centres_xyz, dtype=np.float64) @ r  # rows: (R^T c)^T
    g = np.arange(size) - size // 2
    img = np.zeros((size, size))
    amp = math.sqrt(2 * math.pi) * sigma
    for cx, cy, _ in p:
        gx = np.exp(-((g - cx) ** 2) / (2 * sigma**2))
        gy = np.exp(-((g - cy) ** 2) / (2 * sigma**2))
        img += amp * np.outer(gy, gx)
    return img
