"""Drop-in ``core_refine_template`` running on the GB300 CUDA kernels.

Same arguments and returned keys as Leopard-EM's
``leopard_em.backend.core_refine_template.core_refine_template``
(backend/core_refine_template.py:33-202).  The per-particle Python loop with
per-batch host synchronisation (:447-473, :678-751) becomes one C-ABI call per
group of particles: every particle's CTF stack, offset batches, correlograms,
z-scores and strict '>' best-so-far updates stay on the device; the host only
decodes the winning flat index and composes the Euler angles (:503-551).
"""

from __future__ import annotations

import ctypes
import warnings

import torch

from .. import rotations as rot
from .._native import check, lib
from .._native import RefineProblem, CtfParams


def _device(device) -> torch.device:
    from .core_match_template import _single_cuda_device

    return _single_cuda_device(device)


def _ctf_params(ctf_kwargs: dict) -> CtfParams:
    for key in ("even_zernikes", "odd_zernikes", "mag_matrix"):
        if ctf_kwargs.get(key) is not None:
            raise ValueError(f"ctf_kwargs[{key!r}] is not supported by leopard_em_gb300")
    return CtfParams(
        voltage_kv=float(ctf_kwargs["voltage"]),
        spherical_aberration_mm=float(ctf_kwargs["spherical_aberration"]),
        amplitude_contrast=float(ctf_kwargs["amplitude_contrast_ratio"]),
        b_factor=float(ctf_kwargs["ctf_B_factor"]),
        phase_shift_deg=float(ctf_kwargs["phase_shift"]),
        pixel_size=float(ctf_kwargs["pixel_size"]),
    )


def refine_particles_device(particle_stack_dft, template_dft, euler_angles, euler_angle_offsets, defocus_offsets,
                            defocus_u, defocus_v, defocus_angle, pixel_size_offsets, corr_mean, corr_std, ctf_kwargs,
                            projective_filters, device, batch_size=32, max_correlograms_per_call=16384):
    """Run the local grid for every particle; returns raw per-particle device
    results (best z, its batch's max cc, flat index, batch start, batch length)."""
    dev = _device(device)
    N, H, wc_img = particle_stack_dft.shape
    W = 2 * (wc_img - 1)
    d = template_dft.shape[0]
    K = int(euler_angle_offsets.shape[0])
    D, C = int(defocus_offsets.shape[0]), int(pixel_size_offsets.shape[0])
    B = int(batch_size)
    if B < 1:
        raise ValueError("batch_size must be >= 1")
    # an offset batch never needs more slots than there are offsets: with few
    # offsets (e.g. one starting pose) more particles then share each call
    # (one batch either way, so the tie order is unchanged)
    B = max(1, min(B, K))
    crop_h, crop_w = H - d + 1, W - d + 1
    if tuple(corr_mean.shape) != (N, crop_h, crop_w) or tuple(corr_std.shape) != (N, crop_h, crop_w):
        raise ValueError(f"corr_mean / corr_std must be (N, {crop_h}, {crop_w})")
    if tuple(projective_filters.shape) != (N, d, d // 2 + 1):
        raise ValueError("projective_filters must be (N, d, d//2+1)")
    prm = _ctf_params(ctf_kwargs)
    per_call = max(1, min(N, max_correlograms_per_call // max(1, C * D * B)))
    L = lib()
    out = {k: torch.empty(N, dtype=dt, device=dev) for k, dt in
           [("z", torch.float32), ("cc", torch.float32), ("flat", torch.int32), ("o0", torch.int32),
            ("nb", torch.int32)]}
    with torch.cuda.device(dev):
        s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        f32 = dict(device=dev, dtype=torch.float32)
        tdft = template_dft.to(dev, torch.complex64).contiguous()
        offs = euler_angle_offsets.to(**f32).contiguous()
        dfo = defocus_offsets.to(**f32).contiguous()
        pxo = pixel_size_offsets.to(**f32).contiguous()
        ws = None
        for a in range(0, N, per_call):
            b = min(N, a + per_call)
            prob = RefineProblem(H, W, d, C, D, K, B, b - a)
            if not L.lgb_refine_supported(ctypes.byref(prob)):
                raise ValueError(f"unsupported refinement shape: crop {H}x{W}, template {d}")
            need = ctypes.c_size_t(0)
            check(L.lgb_refine_workspace_size(ctypes.byref(prob), ctypes.byref(need)), "refine workspace")
            if ws is None or ws.numel() < need.value:
                ws = torch.empty(int(need.value), dtype=torch.uint8, device=dev)
            args = [
                particle_stack_dft[a:b].to(dev, torch.complex64).contiguous(),
                euler_angles[a:b].to(**f32).contiguous(),
                defocus_u[a:b].to(**f32).contiguous(),
                defocus_v[a:b].to(**f32).contiguous(),
                defocus_angle[a:b].to(**f32).contiguous(),
                corr_mean[a:b].to(**f32).contiguous(),
                corr_std[a:b].to(**f32).contiguous(),
                projective_filters[a:b].to(**f32).contiguous(),
            ]
            ps, eul, du, dv, dang, cm, cs_, pf = args
            check(
                L.lgb_refine_search(
                    ctypes.byref(prob), ctypes.byref(prm), ps.data_ptr(), tdft.data_ptr(), eul.data_ptr(),
                    offs.data_ptr(), du.data_ptr(), dv.data_ptr(), dang.data_ptr(), dfo.data_ptr(), pxo.data_ptr(),
                    cm.data_ptr(), cs_.data_ptr(), pf.data_ptr(), out["z"][a:b].data_ptr(),
                    out["cc"][a:b].data_ptr(), out["flat"][a:b].data_ptr(), out["o0"][a:b].data_ptr(),
                    out["nb"][a:b].data_ptr(), ws.data_ptr(), ws.numel(), s),
                "lgb_refine_search",
            )
    return out


def core_refine_template(
    particle_stack_dft: torch.Tensor,
    template_dft: torch.Tensor,
    euler_angles: torch.Tensor,
    euler_angle_offsets: torch.Tensor,
    defocus_offsets: torch.Tensor,
    defocus_u: torch.Tensor,
    defocus_v: torch.Tensor,
    defocus_angle: torch.Tensor,
    pixel_size_offsets: torch.Tensor,
    corr_mean: torch.Tensor,
    corr_std: torch.Tensor,
    ctf_kwargs: dict,
    projective_filters: torch.Tensor,
    device: torch.device | list[torch.device],
    batch_size: int = 32,
    num_cuda_streams: int = 1,
    mag_matrix: torch.Tensor | None = None,
) -> dict[str, torch.Tensor]:
    """Refine orientations, defoci and pixel sizes of a particle stack.

    See leopard_em.backend.core_refine_template.core_refine_template; the
    returned dictionary has the same keys (CPU tensors).
    """
    if mag_matrix is not None:
        raise ValueError("anisotropic magnification (mag_matrix) is not supported by leopard_em_gb300")
    if num_cuda_streams > 1:
        warnings.warn("num_cuda_streams is ignored: one fused kernel sequence per particle group", stacklevel=2)
    raw = refine_particles_device(particle_stack_dft, template_dft, euler_angles, euler_angle_offsets,
                                  defocus_offsets, defocus_u, defocus_v, defocus_angle, pixel_size_offsets, corr_mean,
                                  corr_std, ctf_kwargs, projective_filters, device, batch_size)
    raw = {k: v.cpu() for k, v in raw.items()}
    return decode_refine_results(raw, particle_stack_dft.shape, template_dft.shape[0], euler_angles,
                                 euler_angle_offsets, defocus_offsets, pixel_size_offsets)


def decode_refine_results(raw, stack_shape, d, euler_angles, euler_angle_offsets, defocus_offsets,
                          pixel_size_offsets):
    """Flat index -> (offsets, position, angle index); Euler composition and
    wrapping as core_refine_template.py:503-551 and :180-191."""
    N, H, wc_img = stack_shape
    W = 2 * (wc_img - 1)
    crop_w = W - d + 1
    D, C = int(defocus_offsets.shape[0]), int(pixel_size_offsets.shape[0])
    offs = euler_angle_offsets.cpu().to(torch.float32)
    dfo = defocus_offsets.cpu().to(torch.float32)
    pxo = pixel_size_offsets.cpu().to(torch.float32)
    flat = raw["flat"].long()
    nb = raw["nb"].long().clamp_min(1)
    ok = flat >= 0
    f = flat.clamp_min(0)
    n_cpp = C * D * nb
    c = f % n_cpp
    pix = f // n_cpp
    y = torch.where(ok, pix // crop_w, torch.zeros_like(pix))
    x = torch.where(ok, pix % crop_w, torch.zeros_like(pix))
    cs_idx = c // (D * nb)
    df_idx = (c // nb) % D
    a_idx = c % nb
    angle_idx = torch.where(ok, raw["o0"].long() + a_idx, torch.zeros_like(a_idx))
    off_angles = torch.where(ok[:, None], offs[angle_idx], torch.zeros(N, 3))
    df_off = torch.where(ok, dfo[df_idx], torch.zeros(N))
    px_off = torch.where(ok, pxo[cs_idx], torch.zeros(N))
    eul = rot.combine_euler_angles(off_angles.double(), euler_angles.cpu().double()).to(torch.float32)
    eul[:, 0] = torch.where(eul[:, 0] < 0, eul[:, 0] + 360, eul[:, 0])
    eul[:, 1] = torch.where(eul[:, 1] < 0, eul[:, 1] + 180, eul[:, 1])
    eul[:, 2] = torch.where(eul[:, 2] < 0, eul[:, 2] + 360, eul[:, 2])
    return {
        "refined_cross_correlation": raw["cc"].to(torch.float32),
        "refined_z_score": raw["z"].to(torch.float32),
        "refined_euler_angles": eul,
        "refined_defocus_offset": df_off,
        "refined_pixel_size_offset": px_off,
        "refined_pos_y": y - (H - d + 1) // 2,
        "refined_pos_x": x - (W - d + 1) // 2,
        "angle_idx": angle_idx,
    }


def cross_correlate_particle_stack(
    particle_stack_dft: torch.Tensor,
    template_dft: torch.Tensor,
    rotation_matrices: torch.Tensor,
    projective_filters: torch.Tensor,
    mode: str = "valid",
    batch_size: int = 1024,
    mag_matrix: torch.Tensor | None = None,
    device=None,
) -> torch.Tensor:
    """Cross-correlate each particle with the template projected at its own
    rotation (core_refine_template.py:771-895): returns (N, H-h+1, W-w+1)
    for mode "valid", (N, H, W) for "same", on the particles' device (the
    work runs on ``device`` or, for CPU inputs, the current CUDA device)."""
    if mag_matrix is not None:
        raise ValueError("anisotropic magnification (mag_matrix) is not supported by leopard_em_gb300")
    if mode not in ("valid", "same"):
        raise ValueError(f"Invalid mode: {mode}. Must be 'valid' or 'same'.")
    N, H, wc = particle_stack_dft.shape
    W = 2 * (wc - 1)
    d = int(template_dft.shape[0])
    if tuple(template_dft.shape) != (d, d, d // 2 + 1):
        raise ValueError("template_dft must be (d, d, d//2+1)")
    if tuple(rotation_matrices.shape) != (N, 3, 3) or tuple(projective_filters.shape) != (N, d, d // 2 + 1):
        raise ValueError("rotation_matrices must be (N, 3, 3) and projective_filters (N, d, d//2+1)")
    dev = _device(device if device is not None else
                  (particle_stack_dft.device if particle_stack_dft.is_cuda else "cuda"))
    L = lib()
    if not L.lgb_xcorr_stack_supported(H, W, d):
        raise ValueError(f"unsupported shape: particles {H}x{W}, template {d}")
    group = max(1, min(N, N if batch_size == -1 else int(batch_size)))
    m = 0 if mode == "valid" else 1
    out_shape = (N, H - d + 1, W - d + 1) if m == 0 else (N, H, W)
    with torch.cuda.device(dev):
        s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        need = ctypes.c_size_t(0)
        check(L.lgb_xcorr_stack_workspace_size(group, H, W, d, m, ctypes.byref(need)), "xcorr workspace")
        ws = torch.empty(int(need.value), dtype=torch.uint8, device=dev)
        ps = particle_stack_dft.to(dev, torch.complex64).contiguous()
        tdft = template_dft.to(dev, torch.complex64).contiguous()
        rot = rotation_matrices.to(dev, torch.float32).contiguous()
        pf = projective_filters.to(dev, torch.float32).contiguous()
        out = torch.empty(out_shape, dtype=torch.float32, device=dev)
        check(L.lgb_xcorr_stack(N, group, H, W, d, m, ps.data_ptr(), tdft.data_ptr(), rot.data_ptr(), pf.data_ptr(),
                                out.data_ptr(), ws.data_ptr(), ws.numel(), s), "lgb_xcorr_stack")
    return out.to(particle_stack_dft.device)
