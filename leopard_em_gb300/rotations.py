"""ZYZ Euler-angle helpers for the host-side refinement epilogue (FP64).

The published intrinsic Z-Y-Z convention: R = Rz(phi) @ Ry(theta) @ Rz(psi);
inverse theta = acos(R22), phi = atan2(R12, R02), psi = atan2(R21, -R20)
(the conventions of roma's euler_to_rotmat / rotmat_to_euler with "ZYZ",
which Leopard-EM uses at backend/utils.py:25-54).
"""

from __future__ import annotations

import torch


def euler_zyz_to_rotmat(euler_deg: torch.Tensor) -> torch.Tensor:
    a = torch.deg2rad(euler_deg.to(torch.float64))
    phi, theta, psi = a[..., 0], a[..., 1], a[..., 2]
    cp, sp, ct, st, cs, ss = phi.cos(), phi.sin(), theta.cos(), theta.sin(), psi.cos(), psi.sin()
    r = torch.stack([
        cp * ct * cs - sp * ss, -cp * ct * ss - sp * cs, cp * st,
        sp * ct * cs + cp * ss, -sp * ct * ss + cp * cs, sp * st,
        -st * cs, st * ss, ct,
    ], dim=-1)
    return r.reshape(*euler_deg.shape[:-1], 3, 3)


def rotmat_to_euler_zyz(R: torch.Tensor) -> torch.Tensor:
    R = R.to(torch.float64)
    theta = torch.acos(torch.clamp(R[..., 2, 2], -1.0, 1.0))
    phi = torch.atan2(R[..., 1, 2], R[..., 0, 2])
    psi = torch.atan2(R[..., 2, 1], -R[..., 2, 0])
    return torch.rad2deg(torch.stack([phi, theta, psi], dim=-1))


def combine_euler_angles(angle_a: torch.Tensor, angle_b: torch.Tensor) -> torch.Tensor:
    """Euler angles of R(a) @ R(b)."""
    return rotmat_to_euler_zyz(euler_zyz_to_rotmat(angle_a) @ euler_zyz_to_rotmat(angle_b))
