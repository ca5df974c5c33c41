"""CPU restatement of Leopard-EM's z-score peak picking (test infrastructure).

Follows ``analysis/zscore_metric.py:14-41`` (gaussian_noise_zscore_cutoff),
``:43-84`` (find_peaks_from_zscore) and ``analysis/utils.py:6-50``
(filter_peaks_by_distance): candidates above the cutoff in row-major order,
sorted by value descending, walked in order; a candidate already marked is
skipped, otherwise it is picked and every candidate closer than the
threshold (torch.norm of the float coordinate difference) is marked.  The
sort here is stable, so equal values keep row-major order.
"""

from __future__ import annotations

import numpy as np
import torch
from scipy.special import erfcinv


def gaussian_noise_zscore_cutoff(num_ccg: int, false_positives: float = 1.0) -> float:
    """zscore_metric.py:14-41."""
    return float(erfcinv(2.0 * false_positives / num_ccg) * np.sqrt(2.0))


def filter_peaks_by_distance(peak_values: torch.Tensor, peak_locations: torch.Tensor,
                             distance_threshold: float) -> torch.Tensor:
    """utils.py:6-50 (stable descending sort)."""
    peak_values, order = torch.sort(peak_values, descending=True, stable=True)
    loc = peak_locations[order]
    taken = torch.zeros(loc.shape[0], dtype=torch.bool)
    picked = []
    locf = loc.float()
    for i in range(loc.shape[0]):
        if taken[i]:
            continue
        picked.append(loc[i])
        dist = torch.norm(locf - locf[i], dim=1)
        taken |= dist < distance_threshold
    if not picked:
        return torch.zeros((0, 2), dtype=torch.long)
    return torch.stack(picked)


def find_peaks_from_zscore(zscore_map: torch.Tensor, zscore_cutoff: float, mask_radius: float = 5.0):
    """zscore_metric.py:43-84: (pos_y, pos_x) in descending order of z."""
    peaks = torch.nonzero(zscore_map > zscore_cutoff, as_tuple=False)
    if peaks.shape[0] == 0:
        return torch.tensor([], dtype=torch.long), torch.tensor([], dtype=torch.long)
    values = zscore_map[tuple(peaks.t())]
    picked = filter_peaks_by_distance(values, peaks, mask_radius)
    return picked[:, 0], picked[:, 1]
