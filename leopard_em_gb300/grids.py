"""Orientation grids (inputs to the search and the refinement).

``uniform_euler_grid`` covers SO(3) for the whole-orientation search;
``local_euler_offsets`` samples a neighbourhood of the identity for the local
refinement.  Both return ZYZ Euler angles in degrees, float32 (N, 3).
"""

from __future__ import annotations

import math

import numpy as np
import torch


def uniform_euler_grid(out_of_plane_step: float, in_plane_step: float) -> torch.Tensor:
    """(N, 3) ZYZ Euler angles in degrees covering SO(3).

    theta in [0, 180] every ``out_of_plane_step``; at each theta, phi spaced by
    out_of_plane_step / sin(theta) over [0, 360); psi every ``in_plane_step``
    over [0, 360).  ~ 4 pi / step^2 directions times 360 / psi_step rotations.
    """
    blocks = []
    n_theta = int(round(180.0 / out_of_plane_step))
    psis = np.arange(0.0, 360.0 - 1e-9, in_plane_step)
    for it in range(n_theta + 1):
        theta = min(180.0, it * out_of_plane_step)
        n_phi = max(1, int(round(360.0 * math.sin(math.radians(theta)) / out_of_plane_step)))
        phis = np.arange(n_phi) * (360.0 / n_phi)
        ph, ps = np.meshgrid(phis, psis, indexing="ij")
        blocks.append(np.stack([ph.ravel(), np.full(ph.size, theta), ps.ravel()], axis=1))
    return torch.tensor(np.concatenate(blocks), dtype=torch.float32)


def local_euler_offsets(out_of_plane_range: float, out_of_plane_step: float, in_plane_range: float,
                        in_plane_step: float) -> torch.Tensor:
    """(K, 3) ZYZ offsets around the identity for local refinement.

    Tilt directions on rings theta = 0, step, 2*step, ... <= range, each ring
    with round(2*pi*sin(theta)/step) azimuths phi (a pure tilt is
    (phi, theta, -phi)), combined with in-plane offsets psi in
    [-in_plane_range, in_plane_range] every in_plane_step.
    """
    rows = []
    n_t = int(math.floor(out_of_plane_range / out_of_plane_step + 1e-9))
    psis = np.arange(-in_plane_range, in_plane_range + 1e-9, in_plane_step)
    for it in range(n_t + 1):
        theta = it * out_of_plane_step
        n_phi = 1 if it == 0 else max(1, int(round(2 * math.pi * math.sin(math.radians(theta))
                                                    / math.radians(out_of_plane_step))))
        for ip in range(n_phi):
            phi = ip * 360.0 / n_phi
            for psi in psis:
                rows.append((phi, theta, -phi + psi))
    return torch.tensor(rows, dtype=torch.float32)


