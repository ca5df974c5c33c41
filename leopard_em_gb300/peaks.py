"""Peak picking on the z-score map, on the device.

Same functions and results as Leopard-EM's ``analysis/zscore_metric.py``
(``gaussian_noise_zscore_cutoff`` :14-41, ``find_peaks_from_zscore`` :43-84,
``extract_peaks_and_statistics_zscore`` :87-166) with the greedy distance
suppression of ``analysis/utils.py:6-50`` computed by ``lgb_peaks_find``
(rounds of one kernel over the map instead of a host loop over the sorted
candidates).  Equal z values rank in row-major order.
"""

from __future__ import annotations

import ctypes
import math
import warnings
from typing import NamedTuple, Optional

import torch

from ._native import check, lib


class MatchTemplatePeaks(NamedTuple):
    """Peak positions and per-peak statistics (match_template_peaks.py:9-22)."""

    pos_y: torch.Tensor
    pos_x: torch.Tensor
    mip: torch.Tensor
    scaled_mip: torch.Tensor
    psi: torch.Tensor
    theta: torch.Tensor
    phi: torch.Tensor
    relative_defocus: torch.Tensor
    correlation_mean: torch.Tensor
    correlation_variance: torch.Tensor
    total_correlations: int


def gaussian_noise_zscore_cutoff(num_ccg: int, false_positives: float = 1.0) -> float:
    """z cutoff with at most ``false_positives`` expected false peaks among
    ``num_ccg`` Gaussian samples: sqrt(2) * erfcinv(2 fp / num_ccg)."""
    from scipy.special import erfcinv  # pylint: disable=no-name-in-module

    return float(erfcinv(2.0 * false_positives / num_ccg) * math.sqrt(2.0))


def find_peaks_from_zscore(zscore_map: torch.Tensor, zscore_cutoff: float, mask_radius: float = 5.0,
                           device=None, max_rounds: int = 4096) -> tuple[torch.Tensor, torch.Tensor]:
    """(pos_y, pos_x) of the picked peaks, in descending order of z (CPU
    long tensors, like the reference)."""
    from .backend.core_match_template import _single_cuda_device

    if zscore_map.dim() != 2:
        raise ValueError("zscore_map must be 2-D")
    dev = _single_cuda_device(device if device is not None else
                              (zscore_map.device if zscore_map.is_cuda else "cuda"))
    H, W = zscore_map.shape
    L = lib()
    with torch.cuda.device(dev):
        z = zscore_map.to(dev, torch.float32).contiguous()
        nbytes = int(L.lgb_peaks_scratch_size(H, W, max_rounds))
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        cap = 4096
        while True:
            idx = torch.empty(cap, dtype=torch.int32, device=dev)
            n = ctypes.c_int(0)
            rounds = ctypes.c_int(0)
            s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            check(L.lgb_peaks_find(H, W, z.data_ptr(), float(zscore_cutoff), float(mask_radius), max_rounds,
                                   scratch.data_ptr(), nbytes, cap, idx.data_ptr(), ctypes.byref(n),
                                   ctypes.byref(rounds), s), "lgb_peaks_find")
            if n.value <= cap:
                break
            cap = n.value
        flat = idx[: n.value].long()
        vals = z.reshape(-1)[flat]
        # descending z, equal z in row-major order
        order = torch.argsort(flat)
        flat, vals = flat[order], vals[order]
        order = torch.argsort(vals, descending=True, stable=True)
        flat = flat[order].cpu()
    return flat // W, flat % W


def extract_peaks_and_statistics_zscore(mip, scaled_mip, best_psi, best_theta, best_phi, best_defocus,
                                        correlation_average, correlation_variance,
                                        total_correlation_positions: int, false_positives: float = 1.0,
                                        z_score_cutoff: Optional[float] = None, mask_radius: float = 5.0,
                                        device=None) -> MatchTemplatePeaks:
    """Peak positions, heights and poses from search results (zscore_metric.py:87-166)."""
    if z_score_cutoff is None:
        z_score_cutoff = gaussian_noise_zscore_cutoff(mip.numel() * total_correlation_positions, false_positives)
    pos_y, pos_x = find_peaks_from_zscore(scaled_mip, z_score_cutoff, mask_radius, device=device)
    if len(pos_y) == 0:
        warnings.warn("No peaks found using z-score metric.", stacklevel=2)

    def at(t):
        t = torch.as_tensor(t)
        return t[pos_y.to(t.device), pos_x.to(t.device)]

    return MatchTemplatePeaks(
        pos_y=pos_y, pos_x=pos_x, mip=at(mip), scaled_mip=at(scaled_mip), psi=at(best_psi), theta=at(best_theta),
        phi=at(best_phi), relative_defocus=at(best_defocus), correlation_mean=at(correlation_average),
        correlation_variance=at(correlation_variance), total_correlations=total_correlation_positions,
    )
