"""Autotuner for the launch parameters of the whole-orientation search.

Four choices change the speed of ``lgb_match_search`` but not its results at
valid positions (beyond rounding): the orientation of the search (a
transposed micrograph puts its width on the column transform, which pays when
the height has only a slow column kernel, e.g. 5760 rows), the correlation
grid (the FFT lengths; a micrograph may be
zero padded past the smallest compiled grid to a power of two, whose
transforms have the register-fused kernels), the orientation batch B
(correlograms per statistics update: larger batches amortise the
image-spectrum read and the map read-modify-write over more correlograms, at
the cost of a larger intermediate) and the column pass's grid split
(``col_waves``: how many waves of CTAs the correlogram loop is split into).
``tune_search`` times candidates on the caller's own inputs with CUDA events,
by coordinate descent (grid at B = 8, then B on the best grid, then the split),
and caches the winner per device and search shape in a JSON file
(``$LEOPARD_EM_GB300_TUNE_CACHE``, default
``~/.cache/leopard_em_gb300/autotune.json``).  The reference has no
counterpart: its orientation batch is a user setting
(``ComputationalConfigMatch.batch_size``).
"""

from __future__ import annotations

import json
import os
import threading
from dataclasses import asdict, dataclass

import torch

from ._native import lib

CACHE_ENV = "LEOPARD_EM_GB300_TUNE_CACHE"
DEFAULT_BATCHES = (2, 4, 8, 12, 16, 24, 32, 48, 64)
MAX_BATCH_CORRELOGRAMS = 1024  # C * D * B cap: larger batches gain little and hold a big intermediate
DEFAULT_WAVES = (2, 4, 8)
TRANSPOSE_GAIN = 0.9  # a transposed grid must time at most this fraction of the best direct one
_lock = threading.Lock()


@dataclass
class SearchTuning:
    orientation_batch: int
    col_waves: int
    graph_batches: int
    ms_per_orientation: float
    grid_h: int = 0  # 0: the smallest compiled grid
    grid_w: int = 0
    transpose: bool = False  # search the transposed micrograph (grid is then the transposed grid)

    @property
    def grid(self):
        return (self.grid_h, self.grid_w) if self.grid_h > 0 and self.grid_w > 0 else None

    @staticmethod
    def graph_batches_for(batch: int, orientations_per_graph: int = 128) -> int:
        """Batches per CUDA-graph replay: about ``orientations_per_graph`` orientations."""
        return max(1, orientations_per_graph // batch)


def cache_path() -> str:
    return os.environ.get(CACHE_ENV) or os.path.join(os.path.expanduser("~"), ".cache", "leopard_em_gb300",
                                                     "autotune.json")


def _load_cache(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _store_cache(path: str, key: str, value: dict) -> None:
    with _lock:
        data = _load_cache(path)
        data[key] = value
        try:
            os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
            tmp = f"{path}.{os.getpid()}.tmp"
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, path)
        except OSError:
            pass  # a read-only home directory only costs a re-tune


def tuning_key(device: torch.device, grid: tuple[int, int], micrograph: tuple[int, int], template_size: int,
               n_pixel_sizes: int, n_defocus: int) -> str:
    name = torch.cuda.get_device_name(device).replace(" ", "_")
    return (f"{name}/v{lib().lgb_version()}/grid{grid[0]}x{grid[1]}/mic{micrograph[0]}x{micrograph[1]}"
            f"/d{template_size}/C{n_pixel_sizes}/D{n_defocus}")


def _time_candidate(make_search, cand, n_probe: int, repeats: int) -> float:
    search = make_search(cand)
    stream = torch.cuda.current_stream(search.device)
    search.run(0, min(n_probe, cand[1]))  # warm-up: first launches, lazy module loading
    best = float("inf")
    for _ in range(repeats):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        search.run(0, n_probe)
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    del search
    return best / n_probe


def tune_search(image_dft, template_dft, ctf_filters, whitening_filter_template, defocus_values, pixel_values,
                euler_angles, device, batches=DEFAULT_BATCHES, waves=DEFAULT_WAVES, n_probe: int = 192,
                repeats: int = 2, memory_fraction: float = 0.5, use_cache: bool = True,
                tune_grid: bool = True) -> SearchTuning:
    """Pick the grid, orientation batch and column split for this search shape.

    Candidates whose workspace would exceed ``memory_fraction`` of the free
    device memory are skipped.  Probes search the first ``n_probe``
    orientations into scratch maps (the caller's maps are not touched).  With
    ``tune_grid`` False the grid stays the smallest compiled one, which keeps
    the reference's circular correlation in the margin of compiled sizes.
    """
    from .backend.core_match_template import MatchTemplateSearch, _single_cuda_device, grid_candidates, padded_grid
    from ._native import MatchProblem
    import ctypes

    dev = _single_cuda_device(device)
    H, wc = image_dft.shape
    W = 2 * (wc - 1)
    d = int(template_dft.shape[0])
    C, D = int(pixel_values.shape[0]), int(defocus_values.shape[0])
    grids = [(g, False) for g in (grid_candidates(H, W) if tune_grid else [padded_grid(H, W)])]
    if tune_grid and H != W and H % 2 == 0:
        grids += [(g, True) for g in grid_candidates(W, H)]
    key = tuning_key(dev, grids[0][0], (H, W), d, C, D) + ("/grid+T" if tune_grid else "")
    path = cache_path()
    if use_cache:
        hit = _load_cache(path).get(key)
        if hit:
            try:
                return SearchTuning(**hit)
            except TypeError:
                pass
    n_probe = max(1, min(int(n_probe), int(euler_angles.shape[0])))
    with torch.cuda.device(dev):
        # device-resident inputs once, so every candidate shares them
        inputs = dict(
            image_dft=image_dft.to(dev), template_dft=template_dft.to(dev), ctf_filters=ctf_filters.to(dev),
            whitening_filter_template=whitening_filter_template.to(dev), defocus_values=defocus_values.to(dev),
            pixel_values=pixel_values.to(dev), euler_angles=euler_angles[:n_probe].to(dev),
        )
        free = torch.cuda.mem_get_info(dev)[0]

        def make_search(cand):
            (g, tr), b, w = cand
            return MatchTemplateSearch(**inputs, device=dev, orientation_batch_size=b, col_waves=w, grid=g,
                                       transpose=tr)

        def fits(gt, b):
            if C * D * b > MAX_BATCH_CORRELOGRAMS:
                return False
            g, tr = gt
            mh, mw = (W, H) if tr else (H, W)
            p = MatchProblem(g[0], g[1], d, C, D, n_probe, b, mh, mw, 0)
            need = ctypes.c_size_t(0)
            if lib().lgb_match_workspace_size(ctypes.byref(p), ctypes.byref(need)) != 0:
                return False
            return need.value <= memory_fraction * free

        timings = {}

        def time_of(cand):
            if cand not in timings:
                timings[cand] = _time_candidate(make_search, cand, n_probe, repeats)
            return timings[cand]

        w0 = 4 if 4 in waves else waves[0]
        b0 = 8 if 8 in batches else batches[0]
        grid_cands = [g for g in grids if fits(g, b0)] or grids[:1]
        direct = [g for g in grid_cands if not g[1]] or grid_cands[:1]
        best_g = min(direct, key=lambda g: time_of((g, b0, w0)))
        # a transposed search also pays a transposed spectrum per micrograph:
        # take it only when its orientations run clearly faster
        trans = [g for g in grid_cands if g[1]]
        if trans:
            best_t = min(trans, key=lambda g: time_of((g, b0, w0)))
            if time_of((best_t, b0, w0)) < TRANSPOSE_GAIN * time_of((best_g, b0, w0)):
                best_g = best_t
        cands = [b for b in batches if b >= 1 and fits(best_g, b)] or [1]
        best_b = min(cands, key=lambda b: time_of((best_g, b, w0)))
        best_w = min(waves, key=lambda w: time_of((best_g, best_b, w)))
        ms = timings[(best_g, best_b, best_w)]
    tuning = SearchTuning(orientation_batch=best_b, col_waves=best_w,
                          graph_batches=SearchTuning.graph_batches_for(best_b), ms_per_orientation=float(ms),
                          grid_h=best_g[0][0], grid_w=best_g[0][1], transpose=best_g[1])
    if use_cache:
        _store_cache(path, key, asdict(tuning))
    return tuning
