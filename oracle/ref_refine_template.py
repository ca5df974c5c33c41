"""CPU oracle for the plain local-grid refinement (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs may
import this module; the product path never does.

Restates Leopard-EM's ``core_refine_template`` (backend/core_refine_template.py):
  * ``refine_single_particle``  -- ``_core_refine_template_single_thread``
    (:555-767): per-particle CTF stack (ctf_utils.py:19-116), combined filter,
    offset batches composed with the particle's rotation
    (rotmat_composition((R_offset, R_default)) = R_offset @ R_default), the
    batched CPU cross-correlation (cross_correlation.py:287-369), valid crop,
    z = (cc - mean) / std, strict '>' update across batches, decode of the
    flattened (pixel size, defocus, angle) index.
  * ``core_refine_template_cpu`` -- the driver and epilogue (:33-202,
    :480-551): Euler composition (combine_euler_angles, backend/utils.py:25-54),
    wrapping of negative angles, position offset by (H - h + 1) // 2.
Third-party numerics restated from their published definitions (packages not
installed here; parity with them unpinned):
  * torch-ctf ``calculate_ctf_2d``: CTF = -sin(chi),
    chi = -pi*lambda*k^2*df(theta) + pi/2*Cs*lambda^3*k^4 - phase - atan(A/sqrt(1-A^2)),
    df(theta) = defocus + astigmatism*cos(2(theta - angle)), relativistic lambda;
  * torch-fourier-filter ``b_envelope``: exp(-B k^2 / 4);
  * roma ``rotmat_to_euler("ZYZ", degrees=True)``: theta = acos(R22),
    phi = atan2(R12, R02), psi = atan2(R21, -R20).
"""

from __future__ import annotations

import math

import torch

from . import ref_match_template as mt


def electron_wavelength_angstrom(voltage_kv: float) -> float:
    v = voltage_kv * 1e3
    h, m0, e, c = 6.62607015e-34, 9.1093837015e-31, 1.602176634e-19, 299792458.0
    return h / math.sqrt(2 * m0 * e * v * (1 + e * v / (2 * m0 * c * c))) * 1e10


def _freq_grid(shape, pixel_size):
    h, w = shape
    ky = torch.fft.fftfreq(h, dtype=torch.float64)[:, None] / pixel_size
    kx = torch.fft.rfftfreq(w, dtype=torch.float64)[None, :] / pixel_size
    return ky.expand(h, w // 2 + 1), kx.expand(h, w // 2 + 1)


def calculate_ctf_2d(defocus, astigmatism, astigmatism_angle, voltage, spherical_aberration,
                     amplitude_contrast, phase_shift, pixel_size, image_shape):
    """(D, h, w//2+1) CTF on the unshifted rfft grid; defocus/astigmatism in um."""
    ky, kx = _freq_grid(image_shape, pixel_size)
    k2 = kx**2 + ky**2
    ang = torch.atan2(ky, kx)
    lam = electron_wavelength_angstrom(float(voltage))
    cs = float(spherical_aberration) * 1e7
    k5 = math.atan(amplitude_contrast / math.sqrt(1 - amplitude_contrast**2))
    out = []
    for df_um in torch.as_tensor(defocus, dtype=torch.float64).reshape(-1).tolist():
        df = df_um * 1e4 + float(astigmatism) * 1e4 * torch.cos(2 * (ang - math.radians(float(astigmatism_angle))))
        chi = -math.pi * lam * k2 * df + 0.5 * math.pi * cs * lam**3 * k2**2 - math.radians(phase_shift) - k5
        out.append(-torch.sin(chi))
    return torch.stack(out).to(torch.float32)


def b_envelope(B, image_shape, pixel_size):
    ky, kx = _freq_grid(image_shape, pixel_size)
    return torch.exp(-float(B) * (kx**2 + ky**2) / 4).to(torch.float32)


def ctf_filter_stack_full_args(template_shape, defocus_u, defocus_v, defocus_offsets, pixel_size_offsets, **kw):
    """(C, D, h, w//2+1) as calculate_ctf_filter_stack_full_args (ctf_utils.py:19-116)."""
    defocus = defocus_offsets + (float(defocus_u) + float(defocus_v)) / 2
    astig = abs(float(defocus_u) - float(defocus_v)) / 2
    px = kw["pixel_size"]
    cs_values = kw["spherical_aberration"] / torch.pow((px + pixel_size_offsets) / px, 4)
    env = b_envelope(kw["ctf_B_factor"], template_shape, px)
    stack = []
    for cs in cs_values.tolist():
        ctf = calculate_ctf_2d(defocus * 1e-4, astig * 1e-4, kw["astigmatism_angle"], kw["voltage"], cs,
                               kw["amplitude_contrast_ratio"], kw["phase_shift"], px, template_shape)
        stack.append(ctf * env)
    return torch.stack(stack)


def rotmat_to_euler_zyz(R: torch.Tensor) -> torch.Tensor:
    """Intrinsic ZYZ Euler angles (degrees) of rotation matrices (..., 3, 3)."""
    R = R.to(torch.float64)
    theta = torch.acos(torch.clamp(R[..., 2, 2], -1.0, 1.0))
    phi = torch.atan2(R[..., 1, 2], R[..., 0, 2])
    psi = torch.atan2(R[..., 2, 1], -R[..., 2, 0])
    return torch.rad2deg(torch.stack([phi, theta, psi], dim=-1))


def combine_euler_angles(angle_a, angle_b):
    """R(a) @ R(b) back to ZYZ Euler angles (backend/utils.py:25-54)."""
    ra = mt.euler_to_rotmat_zyz(angle_a.reshape(-1, 3), dtype=torch.float64)
    rb = mt.euler_to_rotmat_zyz(angle_b.reshape(-1, 3), dtype=torch.float64)
    return rotmat_to_euler_zyz(ra @ rb).reshape(angle_a.shape)


def refine_single_particle(particle_image_dft, template_dft, euler_angles, euler_angle_offsets, defocus_u,
                           defocus_v, defocus_angle, defocus_offsets, pixel_size_offsets, corr_mean, corr_std,
                           ctf_kwargs, projective_filter, batch_size=32):
    """Plain local grid for one particle (core_refine_template.py:555-767)."""
    img_h, img_w = particle_image_dft.shape
    img_w = 2 * (img_w - 1)
    _, template_h, template_w = template_dft.shape
    template_w = 2 * (template_w - 1)
    crop_h, crop_w = img_h - template_h + 1, img_w - template_w + 1
    best = dict(max_cc=-1e9, max_z_score=-1e9, refined_phi_offset=0.0, refined_theta_offset=0.0,
                refined_psi_offset=0.0, refined_defocus_offset=0.0, refined_pixel_size_offset=0.0,
                refined_pos_y=0, refined_pos_x=0, angle_idx=0)
    default_rot = mt.euler_to_rotmat_zyz(euler_angles.reshape(1, 3)).to(torch.float32)
    kw = dict(ctf_kwargs)
    kw["astigmatism_angle"] = float(defocus_angle)
    ctf = ctf_filter_stack_full_args(kw.pop("template_shape"), defocus_u, defocus_v, defocus_offsets,
                                     pixel_size_offsets, **kw)
    pf = projective_filter[None, None, ...] * ctf
    n_off = euler_angle_offsets.shape[0]
    for i in range(math.ceil(n_off / batch_size)):
        s, e = i * batch_size, min((i + 1) * batch_size, n_off)
        offs = euler_angle_offsets[s:e]
        rot = mt.euler_to_rotmat_zyz(offs).to(torch.float32)
        rot = rot @ default_rot
        cc = mt.cross_correlate_batched_cpu(particle_image_dft, template_dft, rot, pf)
        cc = cc[..., :crop_h, :crop_w]
        z = (cc - corr_mean) / corr_std
        if z.max() > best["max_z_score"]:
            best["max_cc"] = float(cc.max())
            best["max_z_score"] = float(z.max())
            mv, mi = torch.max(z.reshape(-1, crop_h, crop_w), dim=0)
            _, pos = torch.max(mv.reshape(-1), dim=0)
            y, x = int(pos) // crop_w, int(pos) % crop_w
            flat = int(mi[y, x])
            nb = e - s
            px_idx = flat // (len(defocus_offsets) * nb)
            df_idx = (flat // nb) % len(defocus_offsets)
            a_idx = flat % nb
            best.update(refined_phi_offset=float(offs[a_idx, 0]), refined_theta_offset=float(offs[a_idx, 1]),
                        refined_psi_offset=float(offs[a_idx, 2]),
                        refined_defocus_offset=float(defocus_offsets[df_idx]),
                        refined_pixel_size_offset=float(pixel_size_offsets[px_idx]),
                        refined_pos_y=y, refined_pos_x=x, angle_idx=a_idx + s)
    return best


def core_refine_template_cpu(particle_stack_dft, template_dft, euler_angles, euler_angle_offsets, defocus_offsets,
                             defocus_u, defocus_v, defocus_angle, pixel_size_offsets, corr_mean, corr_std,
                             ctf_kwargs, projective_filters, batch_size=32):
    """Driver + epilogue of core_refine_template (:33-202, :480-551) on the CPU."""
    stats = [
        refine_single_particle(particle_stack_dft[i], template_dft, euler_angles[i], euler_angle_offsets,
                               defocus_u[i], defocus_v[i], defocus_angle[i], defocus_offsets, pixel_size_offsets,
                               corr_mean[i], corr_std[i], ctf_kwargs, projective_filters[i], batch_size)
        for i in range(particle_stack_dft.shape[0])
    ]
    n = len(stats)
    eul = torch.empty((n, 3), dtype=torch.float32)
    for i, st in enumerate(stats):
        off = torch.tensor([st["refined_phi_offset"], st["refined_theta_offset"], st["refined_psi_offset"]],
                           dtype=euler_angles.dtype)
        eul[i] = combine_euler_angles(off, euler_angles[i]).to(torch.float32)
    eul[:, 0] = torch.where(eul[:, 0] < 0, eul[:, 0] + 360, eul[:, 0])
    eul[:, 1] = torch.where(eul[:, 1] < 0, eul[:, 1] + 180, eul[:, 1])
    eul[:, 2] = torch.where(eul[:, 2] < 0, eul[:, 2] + 360, eul[:, 2])
    img_h, img_w = particle_stack_dft.shape[1], 2 * (particle_stack_dft.shape[2] - 1)
    th, tw = template_dft.shape[1], 2 * (template_dft.shape[2] - 1)
    pos_y = torch.tensor([s["refined_pos_y"] for s in stats]) - (img_h - th + 1) // 2
    pos_x = torch.tensor([s["refined_pos_x"] for s in stats]) - (img_w - tw + 1) // 2
    return {
        "refined_cross_correlation": torch.tensor([s["max_cc"] for s in stats]),
        "refined_z_score": torch.tensor([s["max_z_score"] for s in stats]),
        "refined_euler_angles": eul,
        "refined_defocus_offset": torch.tensor([s["refined_defocus_offset"] for s in stats]),
        "refined_pixel_size_offset": torch.tensor([s["refined_pixel_size_offset"] for s in stats]),
        "refined_pos_y": pos_y,
        "refined_pos_x": pos_x,
        "angle_idx": torch.tensor([s["angle_idx"] for s in stats]),
    }


def cross_correlate_particle_stack_cpu(particle_stack_dft, template_dft, rotation_matrices, projective_filters,
                                       mode="valid"):
    """core_refine_template.py:771-895 (no mag_matrix): per particle the slice
    at its rotation, ifftshift rows, DC 0, contrast flip, x filter, irfft2,
    ifftshift, normalisation for the particle size, padded rfft, particle *
    conj(projection) (no DC zeroing), irfft2, crop (utils/cross_correlation.py:8-40)."""
    N, H, wc = particle_stack_dft.shape
    W = 2 * (wc - 1)
    d = template_dft.shape[0]
    fs = mt.extract_central_slices_rfft_3d(template_dft, rotation_matrices)
    fs = torch.fft.ifftshift(fs, dim=(-2,))
    fs[..., 0, 0] = 0 + 0j
    fs = fs * -1
    fs = fs * projective_filters
    proj = torch.fft.irfftn(fs, dim=(-2, -1))
    proj = torch.fft.ifftshift(proj, dim=(-2, -1))
    proj = mt.normalize_template_projection(proj, (d, d), (H, W))
    pdft = torch.fft.rfftn(proj, dim=(-2, -1), s=(H, W))
    cc = torch.fft.irfftn(particle_stack_dft * pdft.conj(), dim=(-2, -1))
    if mode == "valid":
        cc = cc[:, : H - d + 1, : W - d + 1]
    elif mode != "same":
        raise ValueError(mode)
    return cc
