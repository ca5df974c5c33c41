"""Whole-orientation search over many micrographs of uneven sizes.

Leopard-EM searches one micrograph per ``core_match_template`` call
(backend/core_match_template.py:146-363), and a program loops over
micrographs on the host.  Here one call walks every micrograph in turn on one
CUDA stream: each micrograph's search runs on its own correlation grid (the
next compiled FFT lengths, or a larger compiled grid whose transforms are
faster, zero padded), with the grid, orientation batch and column split chosen
by the autotuner (cached per shape, so micrographs of a repeated size reuse
the choice), and the orientation batches replayed as CUDA graphs
(``lgb_match_search_graph``).  A micrograph whose height has only a slow
column transform may run transposed (the autotuner times both orientations;
``core_match_template.transposed_template_dft``).
The host enqueues everything without waiting; per-micrograph device times come
from CUDA events between micrographs.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import torch

from .. import autotune
from .core_match_template import (MatchTemplateSearch, _single_cuda_device, padded_grid, transposed_euler_angles,
                                  transposed_template_dft)

PER_MICROGRAPH_KEYS = ("image_dft", "ctf_filters", "whitening_filter_template", "defocus_values", "pixel_values")


@dataclass
class BatchedSearchReport:
    """Device milliseconds per micrograph (set-up + search + finalize) and the
    launch parameters each micrograph ran with."""

    ms: list[float] = field(default_factory=list)
    grids: list[tuple[int, int]] = field(default_factory=list)
    tunings: list[autotune.SearchTuning] = field(default_factory=list)

    def percentile(self, q: float) -> float:
        if not self.ms:
            return float("nan")
        return float(torch.quantile(torch.tensor(self.ms, dtype=torch.float64), q / 100.0))


def match_template_batch(micrographs, template_dft, euler_angles, device, orientation_range=None, tune: bool = True,
                         orientation_batch_size: int = 8, use_graphs: bool = True, to_cpu: bool = True,
                         tune_cache: bool = True):
    """Search every micrograph over the same template and orientation set.

    ``micrographs``: a sequence of dicts with the per-micrograph arguments of
    ``core_match_template`` (``image_dft``, ``ctf_filters``,
    ``whitening_filter_template``, ``defocus_values``, ``pixel_values``).
    ``orientation_range`` = (begin, end) restricts the search to part of the
    orientation set (all micrographs alike); the statistics still count only
    the correlograms searched.  Returns (results, report): one
    ``core_match_template`` result dict per micrograph (maps H x W of that
    micrograph) and a ``BatchedSearchReport``.
    """
    dev = _single_cuda_device(device)
    n_o = int(euler_angles.shape[0])
    begin, end = (0, n_o) if orientation_range is None else (int(orientation_range[0]), int(orientation_range[1]))
    if not 0 <= begin <= end <= n_o:
        raise ValueError(f"orientation range [{begin}, {end}) outside [0, {n_o})")
    for i, m in enumerate(micrographs):
        missing = [k for k in PER_MICROGRAPH_KEYS if k not in m]
        if missing:
            raise ValueError(f"micrograph {i} is missing {missing}")
    report = BatchedSearchReport()
    results = []
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev)
        tdft = template_dft.to(dev, torch.complex64).contiguous()
        eul = euler_angles.to(dev, torch.float32).contiguous()
        events = []
        pending = []
        tdft_t = eul_t = None  # template and rotations of the transposed frame, made once
        for m in micrographs:
            H, wc = m["image_dft"].shape
            if tune:
                t = autotune.tune_search(m["image_dft"], tdft, m["ctf_filters"], m["whitening_filter_template"],
                                         m["defocus_values"], m["pixel_values"], eul, dev, use_cache=tune_cache)
            else:
                b = int(orientation_batch_size)
                t = autotune.SearchTuning(b, 0, autotune.SearchTuning.graph_batches_for(b), float("nan"))
            tr = bool(getattr(t, "transpose", False))
            grid = t.grid or (padded_grid(2 * (wc - 1), H) if tr else padded_grid(H, 2 * (wc - 1)))
            if tr and tdft_t is None:
                tdft_t = transposed_template_dft(tdft)
                eul_t = transposed_euler_angles(eul).to(dev)
            a = torch.cuda.Event(enable_timing=True)
            z = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            search = MatchTemplateSearch(m["image_dft"], tdft, m["ctf_filters"], m["whitening_filter_template"],
                                         m["defocus_values"], m["pixel_values"], eul, dev,
                                         orientation_batch_size=t.orientation_batch,
                                         graph_batches=t.graph_batches if use_graphs else 0, col_waves=t.col_waves,
                                         grid=grid, transpose=tr, transposed_template=tdft_t if tr else None,
                                         transposed_euler=eul_t if tr else None)
            search.run(begin, end)
            res = search.result(to_cpu=False)
            z.record(stream)
            del search
            events.append((a, z))
            pending.append(res)
            report.grids.append(grid)
            report.tunings.append(t)
        stream.synchronize()
        for (a, z), res in zip(events, pending):
            report.ms.append(a.elapsed_time(z))
            results.append({k: (v.cpu() if to_cpu and isinstance(v, torch.Tensor) else v) for k, v in res.items()})
    return results, report
