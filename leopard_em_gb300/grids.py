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


def _arange_closed(lo: float, hi: float, step: float) -> np.ndarray:
    """lo, lo + step, ... <= hi (both ends of a bounded window included)."""
    if step <= 0:
        return np.array([lo])
    n = int(math.floor((hi - lo) / step + 1e-9))
    return lo + step * np.arange(n + 1)


def symmetry_ranges(group: str, order: int = 1) -> tuple[float, float, float, float, float, float]:
    """(phi_min, phi_max, theta_min, theta_max, psi_min, psi_max) in degrees of
    the asymmetric unit searched for a template of the given point group.

    Cn: an n-fold axis along z makes rotations psi and psi + 360/n equivalent
    (R Rz(360/n) = R for the template), so psi covers [0, 360/n).  Dn adds the
    two-fold axes perpendicular to z, which map theta to 180 - theta: theta
    covers [0, 90].  The polyhedral groups (T, O, I) have no range form of
    their asymmetric unit and are not supported.  Used where the reference
    calls torch-so3's get_symmetry_ranges (config/orientation_search.py:143-147).
    """
    g = group.upper()
    if order < 1:
        raise ValueError(f"symmetry order must be >= 1, got {order}")
    if g == "C":
        return 0.0, 360.0, 0.0, 180.0, 0.0, 360.0 / order
    if g == "D":
        return 0.0, 360.0, 0.0, 90.0, 0.0, 360.0 / order
    raise ValueError(f"symmetry group '{group}' is not supported (C and D only)")


def uniform_euler_angles(psi_step: float, theta_step: float, phi_min: float = 0.0, phi_max: float = 360.0,
                         theta_min: float = 0.0, theta_max: float = 180.0, psi_min: float = 0.0,
                         psi_max: float = 360.0, base_grid_method: str = "uniform",
                         psi_periodic: bool | None = None) -> torch.Tensor:
    """(N, 3) ZYZ Euler angles (phi, theta, psi) in degrees over the given ranges.

    The construction behind ``OrientationSearchConfig.euler_angles``
    (config/orientation_search.py:130-170, torch-so3's get_uniform_euler_angles):
    theta rings every ``theta_step`` over [theta_min, theta_max] (both ends);
    "uniform" places max(1, round((phi_max - phi_min) sin(theta) / theta_step))
    azimuths on a ring, so directions are spaced about ``theta_step`` apart on
    the sphere; "cartesian" uses ``theta_step`` for phi as well, independent of
    theta; psi every ``psi_step``.  A full-circle phi or psi range (360 degrees)
    is periodic and excludes its end point; a narrower range is a closed
    window.  ``psi_periodic`` forces the psi rule (a symmetry group's psi
    range [0, 360/n) is periodic: psi = 360/n is psi = 0).  Over the full
    ranges this is ``uniform_euler_grid``.
    """
    if base_grid_method not in ("uniform", "cartesian"):
        raise ValueError(f"base_grid_method '{base_grid_method}' is not supported (uniform, cartesian)")
    if theta_step <= 0 or psi_step <= 0:
        raise ValueError("theta_step and psi_step must be > 0")
    thetas = _arange_closed(theta_min, theta_max, theta_step)
    psi_span = psi_max - psi_min
    if psi_periodic is None:
        psi_periodic = abs(psi_span - 360.0) < 1e-9
    if psi_periodic:
        psis = psi_min + psi_step * np.arange(int(math.ceil(psi_span / psi_step)) if psi_span > 0 else 1)
        psis = psis[psis < psi_max - 1e-9]
    else:
        psis = _arange_closed(psi_min, psi_max, psi_step)
    phi_span = phi_max - phi_min
    periodic_phi = abs(phi_span - 360.0) < 1e-9
    blocks = []
    for theta in thetas:
        if base_grid_method == "uniform":
            n_phi = max(1, int(round(phi_span * abs(math.sin(math.radians(theta))) / theta_step)))
            if periodic_phi:
                phis = phi_min + np.arange(n_phi) * (phi_span / n_phi)
            else:  # centred cells of a closed window
                phis = phi_min + (np.arange(n_phi) + 0.5) * (phi_span / n_phi)
        else:
            phis = _arange_closed(phi_min, phi_max, theta_step)
            if periodic_phi:
                phis = phis[phis < phi_max - 1e-9]
        ph, ps = np.meshgrid(phis, psis, indexing="ij")
        blocks.append(np.stack([ph.ravel(), np.full(ph.size, theta), ps.ravel()], axis=1))
    return torch.tensor(np.concatenate(blocks), dtype=torch.float32)


def local_high_resolution_angles(coarse_phi_step: float, coarse_theta_step: float, coarse_psi_step: float,
                                 fine_phi_step: float, fine_theta_step: float, fine_psi_step: float,
                                 base_grid_method: str = "uniform") -> torch.Tensor:
    """(K, 3) ZYZ offsets for the local refinement grid of
    ``RefineOrientationConfig.euler_angles_offsets``
    (config/orientation_search.py:256-278, torch-so3's
    get_local_high_resolution_angles).

    Each angle is sampled over [-coarse, +coarse] in steps of its fine step,
    both ends included (the reference's description of the refinement grid).
    "uniform": the out-of-plane pair (phi, theta) is the uniform base grid of
    ``uniform_euler_angles`` restricted to the window -- theta rings every
    fine theta step, each ring with max(1, round(2 coarse_phi |sin theta| /
    fine_theta)) azimuths centred in the phi window; "basic": phi, theta and
    psi as three independent closed ranges.  The reference's test pins
    (psi 1.5/0.5, theta 2.5/1.0, phi 2.5/0.25) to 42 offsets
    (tests/pydantic_models/test_orientation_search.py:179-196); the
    third-party package itself is not installed here, so the offsets beyond
    that count are this restatement's.
    """
    if base_grid_method == "basic":
        phis = _arange_closed(-coarse_phi_step, coarse_phi_step, fine_phi_step)
        thetas = _arange_closed(-coarse_theta_step, coarse_theta_step, fine_theta_step)
        psis = _arange_closed(-coarse_psi_step, coarse_psi_step, fine_psi_step)
        g = np.stack(np.meshgrid(phis, thetas, psis, indexing="ij"), axis=-1).reshape(-1, 3)
        return torch.tensor(g, dtype=torch.float32)
    if base_grid_method != "uniform":
        raise ValueError(f"base_grid_method '{base_grid_method}' is not supported (uniform, basic)")
    return uniform_euler_angles(psi_step=fine_psi_step, theta_step=fine_theta_step, phi_min=-coarse_phi_step,
                                phi_max=coarse_phi_step, theta_min=-coarse_theta_step, theta_max=coarse_theta_step,
                                psi_min=-coarse_psi_step, psi_max=coarse_psi_step, base_grid_method="uniform")


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


