"""Drop-in ``core_match_template`` running on the GB300 CUDA kernels.

Same positional/keyword arguments and returned keys as Leopard-EM's
``leopard_em.backend.core_match_template.core_match_template``
(backend/core_match_template.py:146-363).  One process, one GPU, one CUDA
stream: the reference's worker processes, work queue and per-stream
round-robin (core_match_template.py:283-327, cross_correlation.py:101-142)
become one in-order sequence of fused kernels on the caller's current stream.

Semantics kept from the reference:
  * projective filters = ctf_filters * whitening (core_match_template.py:274);
  * global search index cs*D*N + df*N + orientation (:458-466, :513-520);
  * MIP update with strict '>' per orientation batch, first index wins inside
    a batch (backend/utils.py:241-252);
  * decode and z-score scaling of process_results.py:67-183, including the
    "correlation_variance" key holding the standard deviation.
Deliberate differences:
  * sums and sums of squares accumulate in FP64 (reference: FP32);
  * the last, partial orientation batch is indexed correctly (the reference
    always builds a full-length index vector, :513-520);
  * a micrograph whose height or width is not a compiled FFT length is
    searched on the next compiled grid with zero padding.  Correlations at
    valid positions (y <= H - d, x <= W - d) are those of the unpadded
    search; in the margin the reference's circular wrap-around becomes a
    linear correlation (the manager crops that margin,
    match_template_result.py apply_valid_cropping).
"""

from __future__ import annotations

import ctypes
import warnings

import torch

from .._native import MatchProblem, check, lib


# precision modes of lgb_match_search_precision (0 = the plain FP32 search)
PRECISION_MODES = {"fp32": 0, "bf16x3": 1, "fp16x3": 2}


def _single_cuda_device(device) -> torch.device:
    if isinstance(device, (list, tuple)):
        if len(device) != 1:
            raise ValueError(
                f"leopard_em_gb300 runs on exactly one GPU per call; got {len(device)} devices"
            )
        device = device[0]
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError(f"leopard_em_gb300 needs a CUDA device, got {device}")
    if device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    return device


def _ptr(t: torch.Tensor) -> int:
    """Device address of a tensor handed to the C ABI (dense row-major only)."""
    if not t.is_contiguous():
        raise ValueError(f"tensor of shape {tuple(t.shape)} is not contiguous; the C ABI takes row-major buffers")
    return t.data_ptr()


def grid_candidates(h: int, w: int) -> list[tuple[int, int]]:
    """Compiled grids worth timing for an h x w micrograph: per axis the
    smallest compiled length and the smallest compiled power of two (whose
    transforms have the fastest kernels), smallest grid first."""
    L = lib()
    axes = []
    for n, axis in ((h, 0), (w, 1)):
        c = {int(L.lgb_match_fft_size(int(n), axis))}
        p2 = 1 << max(0, int(n) - 1).bit_length()
        c.add(int(L.lgb_match_fft_size(p2, axis)) if L.lgb_match_fft_size(p2, axis) == p2 else 0)
        axes.append(sorted(x for x in c if x > 0))
    if not axes[0] or not axes[1]:
        raise ValueError(f"no compiled FFT grid holds a {h}x{w} micrograph")
    return sorted(((a, b) for a in axes[0] for b in axes[1]), key=lambda g: (g[0] * g[1], g))


def padded_grid(h: int, w: int) -> tuple[int, int]:
    """Correlation grid for an h x w micrograph: the smallest compiled FFT
    lengths >= h and >= w (equal to (h, w) when both are compiled)."""
    L = lib()
    hp, wp = int(L.lgb_match_fft_size(int(h), 0)), int(L.lgb_match_fft_size(int(w), 1))
    if hp == 0 or wp == 0:
        raise ValueError(f"no compiled FFT grid holds a {h}x{w} micrograph")
    return hp, wp


# ---------------------------------------------------------------------------
# Transposed search.  Searching the transposed micrograph I^T with the template
# volume's x and y axes swapped and every rotation conjugated by that swap
# (R' = S R S, S the x <-> y exchange; a proper rotation again) yields the
# transposed correlograms: the projection of the swapped volume at R' is the
# transposed projection at R, and the cross-correlation of transposed images
# is the transposed cross-correlation.  The statistics maps of the transposed
# search are the transposed maps of the direct search (the orientation index
# of every correlogram is unchanged), so a micrograph whose height has only a
# slow column transform (e.g. 5760) can run on the fused kernels of its width.
# ---------------------------------------------------------------------------
_SWAP_XY = torch.tensor([[0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]], dtype=torch.float64)


def _rotmat_to_euler_zyz_robust(R: torch.Tensor) -> torch.Tensor:
    """ZYZ Euler angles (degrees) of rotations (N, 3, 3), FP64, including
    theta = 0 and 180 (psi = 0 there, phi carries the whole z rotation)."""
    R = R.to(torch.float64)
    theta = torch.acos(torch.clamp(R[:, 2, 2], -1.0, 1.0))
    st = torch.sqrt(R[:, 0, 2] ** 2 + R[:, 1, 2] ** 2)
    regular = st > 1e-9
    phi = torch.where(regular, torch.atan2(R[:, 1, 2], R[:, 0, 2]), torch.zeros_like(theta))
    psi = torch.where(regular, torch.atan2(R[:, 2, 1], -R[:, 2, 0]), torch.zeros_like(theta))
    # theta = 0: R = Rz(phi + psi); theta = pi: R = Rz(phi) diag(-1, 1, -1) Rz(psi)
    top = R[:, 2, 2] > 0
    phi_sing = torch.where(top, torch.atan2(R[:, 1, 0], R[:, 0, 0]), torch.atan2(-R[:, 1, 0], -R[:, 0, 0]))
    phi = torch.where(regular, phi, phi_sing)
    return torch.rad2deg(torch.stack([phi, theta, psi], dim=1))


def transposed_euler_angles(euler_angles: torch.Tensor) -> torch.Tensor:
    """Euler angles of S R S for every orientation (float32)."""
    from ..rotations import euler_zyz_to_rotmat

    R = euler_zyz_to_rotmat(euler_angles.detach().cpu().to(torch.float64))
    S = _SWAP_XY
    return _rotmat_to_euler_zyz_robust(S @ R @ S).to(torch.float32)


def transposed_half_filter(f: torch.Tensor) -> torch.Tensor:
    """A real, Hermitian-even filter (..., d, d//2+1) on the rfft grid, as seen
    in the transposed frame: f'(ky, kx) = f(kx, ky), completing the negative
    kx half by f(-k) = f(k)."""
    d = f.shape[-2]
    i = torch.arange(d, device=f.device)[:, None]
    j = torch.arange(d // 2 + 1, device=f.device)[None, :]
    low = i <= d // 2
    rows = torch.where(low, j, (d - j) % d)
    cols = torch.where(low, i, d - i).expand_as(rows)
    return f[..., rows, cols].contiguous()


def transposed_template_dft(template_dft: torch.Tensor) -> torch.Tensor:
    """Template spectrum (fftshifted rfft layout, d x d x d//2+1) of the volume
    with its x and y axes exchanged."""
    d = template_dft.shape[0]
    v = torch.fft.irfftn(torch.fft.ifftshift(template_dft.to(torch.complex64), dim=(0, 1)), s=(d, d, d))
    v = torch.fft.ifftshift(v, dim=(0, 1, 2)).transpose(1, 2).contiguous()
    t = torch.fft.rfftn(torch.fft.fftshift(v, dim=(0, 1, 2)), dim=(0, 1, 2))
    return torch.fft.fftshift(t, dim=(0, 1)).contiguous()


def transposed_image_dft(image_dft: torch.Tensor) -> torch.Tensor:
    """rfft of the transposed micrograph (H x W -> W x H; H must be even)."""
    H, wc = image_dft.shape
    W = 2 * (wc - 1)
    if H % 2:
        raise ValueError("a transposed search needs an even micrograph height")
    img = torch.fft.irfftn(image_dft.to(torch.complex64), s=(H, W))
    return torch.fft.rfftn(img.transpose(0, 1).contiguous()).contiguous()


class MatchTemplateSearch:
    """Device state of one whole-orientation search over one micrograph.

    Holds the device copies of the inputs, the projective-filter stack, the
    kernels' workspace and the four statistics maps.  ``run(begin, end)``
    correlates an orientation range (callers may split the range to report
    progress); ``result()`` decodes and scales the maps.
    """

    def __init__(
        self,
        image_dft: torch.Tensor,
        template_dft: torch.Tensor,
        ctf_filters: torch.Tensor,
        whitening_filter_template: torch.Tensor,
        defocus_values: torch.Tensor,
        pixel_values: torch.Tensor,
        euler_angles: torch.Tensor,
        device,
        orientation_batch_size: int = 1,
        graph_batches: int = 0,
        col_waves: int = 0,
        grid: tuple[int, int] | None = None,
        precision: str = "fp32",
        transpose: bool = False,
        transposed_template: torch.Tensor | None = None,
        transposed_euler: torch.Tensor | None = None,
    ):
        """``graph_batches`` > 0 replays that many orientation batches per CUDA
        graph launch (``lgb_match_search_graph``); ``col_waves`` sets the column
        pass launch shape (0 = default).  Neither changes any result.
        ``grid`` = (rows, columns) searches on a larger compiled grid than the
        smallest one that holds the micrograph (zero padding; the valid region
        is unchanged, the margin becomes a linear correlation).
        ``precision`` = "bf16x3" / "fp16x3" runs the inverse DFT stages as
        split-precision tensor-core GEMMs (``lgb_match_search_precision``);
        "fp32" (default) is the plain FP32 search.
        ``transpose`` searches the transposed micrograph (see
        ``transposed_template_dft``): ``grid`` is then the transposed grid
        (columns, rows), results and ``maps()`` come back in the micrograph's
        own frame; ``transposed_template`` / ``transposed_euler`` may pass
        precomputed ``transposed_template_dft(template_dft)`` /
        ``transposed_euler_angles(euler_angles)`` (shared by several
        micrographs).  Results at valid positions equal the direct search's to
        rounding (the conjugated rotations are rounded to FP32 Euler angles)."""
        self.device = _single_cuda_device(device)
        self.transpose = bool(transpose)
        self.decode_euler = None
        if self.transpose:
            if precision != "fp32":
                raise ValueError("a transposed search runs the plain FP32 kernels only")
            dev0 = _single_cuda_device(device)
            self.decode_euler = euler_angles.to(dev0, torch.float32).contiguous()
            image_dft = transposed_image_dft(image_dft.to(dev0))
            template_dft = (transposed_template if transposed_template is not None
                            else transposed_template_dft(template_dft.to(dev0)))
            ctf_filters = transposed_half_filter(ctf_filters.to(dev0))
            whitening_filter_template = transposed_half_filter(whitening_filter_template.to(dev0))
            euler_angles = transposed_euler if transposed_euler is not None else transposed_euler_angles(euler_angles)
        if image_dft.dim() != 2 or template_dft.dim() != 3:
            raise ValueError("image_dft must be (H, W//2+1) and template_dft (d, d, d//2+1)")
        H, wc_img = image_dft.shape
        W = 2 * (wc_img - 1)
        d = template_dft.shape[0]
        if tuple(template_dft.shape) != (d, d, d // 2 + 1):
            raise ValueError(f"template_dft must be cubic (d, d, d//2+1), got {tuple(template_dft.shape)}")
        n_cs, n_df = int(pixel_values.shape[0]), int(defocus_values.shape[0])
        if tuple(ctf_filters.shape) != (n_cs, n_df, d, d // 2 + 1):
            raise ValueError(
                f"ctf_filters must be (num_Cs={n_cs}, num_defocus={n_df}, {d}, {d // 2 + 1}), "
                f"got {tuple(ctf_filters.shape)}"
            )
        if tuple(whitening_filter_template.shape) != (d, d // 2 + 1):
            raise ValueError("whitening_filter_template must be (d, d//2+1)")
        if euler_angles.dim() != 2 or euler_angles.shape[1] != 3:
            raise ValueError("euler_angles must be (N, 3)")
        if orientation_batch_size < 1:
            raise ValueError("orientation_batch_size must be >= 1")
        if graph_batches < 0 or col_waves < 0:
            raise ValueError("graph_batches and col_waves must be >= 0")
        if precision not in PRECISION_MODES:
            raise ValueError(f"precision must be one of {sorted(PRECISION_MODES)}, got {precision!r}")
        self.precision_mode = PRECISION_MODES[precision]
        L = lib()
        Hp, Wp = padded_grid(H, W) if grid is None else (int(grid[0]), int(grid[1]))
        if Hp < H or Wp < W:
            raise ValueError(f"grid {Hp}x{Wp} does not hold a {H}x{W} micrograph")
        self.problem = MatchProblem(
            image_h=Hp,
            image_w=Wp,
            template_size=d,
            n_pixel_sizes=n_cs,
            n_defocus=n_df,
            n_orientations=int(euler_angles.shape[0]),
            orientation_batch=int(orientation_batch_size),
            micrograph_h=H,
            micrograph_w=W,
            col_waves=int(col_waves),
        )
        self.graph_batches = int(graph_batches)
        if self.precision_mode and not L.lgb_match_precision_supported(ctypes.byref(self.problem),
                                                                       self.precision_mode):
            raise ValueError(
                f"precision {precision!r} does not support this shape (image {H}x{W}, template {d}, "
                f"{n_cs * n_df * orientation_batch_size} correlograms per batch)"
            )
        if not L.lgb_match_supported(ctypes.byref(self.problem)):
            raise ValueError(
                f"unsupported search shape: image {H}x{W} (grid {Hp}x{Wp}), template {d} "
                "(FFT lengths outside the compiled set)"
            )
        dev = self.device
        with torch.cuda.device(dev):
            stream = torch.cuda.current_stream(dev)
            self._stream = stream
            s = ctypes.c_void_p(stream.cuda_stream)
            self.image_dft = image_dft.to(dev, torch.complex64, non_blocking=True).contiguous()
            if (Hp, Wp) != (H, W):
                # spectrum of the zero-padded micrograph (set-up, once per micrograph)
                img = torch.fft.irfftn(self.image_dft, s=(H, W))
                # (cuFFT returns the 2-D transform with transposed strides)
                self.image_dft = torch.fft.rfftn(torch.nn.functional.pad(img, (0, Wp - W, 0, Hp - H))).contiguous()
                del img
            self.template_dft = template_dft.to(dev, torch.complex64, non_blocking=True).contiguous()
            self.euler_angles = euler_angles.to(dev, torch.float32, non_blocking=True).contiguous()
            self.defocus_values = defocus_values.to(dev, torch.float32, non_blocking=True).contiguous()
            self.pixel_values = pixel_values.to(dev, torch.float32)
            ctf = ctf_filters.to(dev, torch.float32, non_blocking=True).contiguous()
            wf = whitening_filter_template.to(dev, torch.float32, non_blocking=True).contiguous()
            self.projective_filters = torch.empty_like(ctf)
            check(
                L.lgb_match_filters(ctypes.byref(self.problem), _ptr(ctf), _ptr(wf), _ptr(self.projective_filters), s),
                "lgb_match_filters",
            )
            nbytes = ctypes.c_size_t(0)
            if self.precision_mode:
                check(L.lgb_match_precision_workspace_size(ctypes.byref(self.problem), ctypes.byref(nbytes)),
                      "precision workspace size")
            else:
                check(L.lgb_match_workspace_size(ctypes.byref(self.problem), ctypes.byref(nbytes)), "workspace size")
            self.device_status = torch.zeros(1, dtype=torch.int32, device=dev)
            self.workspace = torch.empty(int(nbytes.value), dtype=torch.uint8, device=dev)
            self.mip = torch.empty((Hp, Wp), dtype=torch.float32, device=dev)
            self.best_index = torch.empty((Hp, Wp), dtype=torch.int32, device=dev)
            self.corr_sum = torch.empty((Hp, Wp), dtype=torch.float64, device=dev)
            self.corr_sq_sum = torch.empty((Hp, Wp), dtype=torch.float64, device=dev)
            check(
                L.lgb_match_init_stats(
                    Hp * Wp, _ptr(self.mip), _ptr(self.best_index), _ptr(self.corr_sum), _ptr(self.corr_sq_sum), s
                ),
                "lgb_match_init_stats",
            )
            check(
                L.lgb_match_prepare_image(
                    ctypes.byref(self.problem), _ptr(self.image_dft), _ptr(self.workspace), self.workspace.numel(), s
                ),
                "lgb_match_prepare_image",
            )
        self.shape = (H, W)
        self.grid = (Hp, Wp)
        self.orientations_done = 0

    @property
    def total_projections(self) -> int:
        p = self.problem
        return p.n_orientations * p.n_defocus * p.n_pixel_sizes

    @property
    def searched_projections(self) -> int:
        """Correlograms folded into the maps so far (the mean / std divisor;
        equal to ``total_projections`` once every orientation has run)."""
        p = self.problem
        done = self.orientations_done if self.orientations_done > 0 else p.n_orientations
        return done * p.n_defocus * p.n_pixel_sizes

    def run(self, begin: int = 0, end: int | None = None) -> None:
        """Correlate orientations [begin, end) and fold them into the maps."""
        end = self.problem.n_orientations if end is None else end
        if not 0 <= begin <= end <= self.problem.n_orientations:
            raise ValueError(f"orientation range [{begin}, {end}) outside [0, {self.problem.n_orientations})")
        with torch.cuda.device(self.device):
            s = ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
            if self.precision_mode:
                check(
                    lib().lgb_match_search_precision(
                        ctypes.byref(self.problem), self.precision_mode, _ptr(self.template_dft),
                        _ptr(self.projective_filters), _ptr(self.euler_angles), int(begin), int(end), _ptr(self.mip),
                        _ptr(self.best_index), _ptr(self.corr_sum), _ptr(self.corr_sq_sum), _ptr(self.workspace),
                        self.workspace.numel(), _ptr(self.device_status), s),
                    "lgb_match_search_precision",
                )
                self.orientations_done += end - begin
                return
            if self.graph_batches > 0:
                check(
                    lib().lgb_match_search_graph(
                        ctypes.byref(self.problem), _ptr(self.template_dft), _ptr(self.projective_filters),
                        _ptr(self.euler_angles), int(begin), int(end), self.graph_batches, _ptr(self.mip),
                        _ptr(self.best_index), _ptr(self.corr_sum), _ptr(self.corr_sq_sum), _ptr(self.workspace),
                        self.workspace.numel(), s),
                    "lgb_match_search_graph",
                )
                self.orientations_done += end - begin
                return
            check(
                lib().lgb_match_search(
                    ctypes.byref(self.problem),
                    _ptr(self.template_dft),
                    _ptr(self.projective_filters),
                    _ptr(self.euler_angles),
                    int(begin),
                    int(end),
                    _ptr(self.mip),
                    _ptr(self.best_index),
                    _ptr(self.corr_sum),
                    _ptr(self.corr_sq_sum),
                    _ptr(self.workspace),
                    self.workspace.numel(),
                    s,
                ),
                "lgb_match_search",
            )
        self.orientations_done += end - begin

    def maps(self) -> dict:
        """The four running maps (device tensors, shared with the search; for a
        transposed search, transposed views in the micrograph's frame)."""
        m = {"mip": self.mip, "best_global_index": self.best_index, "correlation_sum": self.corr_sum,
             "correlation_squared_sum": self.corr_sq_sum}
        return {k: v.t() for k, v in m.items()} if self.transpose else m

    def state_dict(self) -> dict:
        """Resumable state (CPU tensors): the four maps and the orientations
        folded so far.  The maps at a batch boundary plus the next orientation
        index are a complete state of the search (the reference has no resume;
        match_template_result.py:51-56 lists it as future work)."""
        p = self.problem
        return {
            "maps": {k: v.cpu() for k, v in self.maps().items()},
            "orientations_done": int(self.orientations_done),
            "problem": {name: int(getattr(p, name)) for name, _ in p._fields_ if name != "col_waves"},
        }

    def load_state_dict(self, state: dict) -> None:
        """Restore a ``state_dict`` taken from a search of the same shape."""
        p = self.problem
        mine = {name: int(getattr(p, name)) for name, _ in p._fields_ if name != "col_waves"}
        mine.pop("orientation_batch")
        theirs = dict(state["problem"])
        theirs.pop("orientation_batch", None)
        if mine != theirs:
            raise ValueError(f"state of a different search shape: {theirs} vs {mine}")
        self.load_maps(state["maps"])
        self.orientations_done = int(state["orientations_done"])

    def load_maps(self, maps: dict) -> None:
        """Replace the running maps, e.g. with the reduction of every rank's maps."""
        tr = (lambda t: t.t()) if self.transpose else (lambda t: t)
        with torch.cuda.device(self.device):
            self.mip.copy_(tr(maps["mip"]))
            self.best_index.copy_(tr(maps["best_global_index"]))
            self.corr_sum.copy_(tr(maps["correlation_sum"]))
            self.corr_sq_sum.copy_(tr(maps["correlation_squared_sum"]))

    def result(self, to_cpu: bool = True) -> dict:
        """Decode indices and compute mean / std / z-score (process_results.py:67-183).

        Maps are H x W (the micrograph), also when the search ran on a padded grid."""
        H, W = self.shape
        Hp, Wp = self.grid
        dev = self.device
        if self.precision_mode:
            status = int(self.device_status.item())
            if status:
                check(status, "device-side status of the search")
        with torch.cuda.device(dev):
            s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            out = {k: torch.empty((Hp, Wp), dtype=torch.float32, device=dev) for k in
                   ("scaled_mip", "best_phi", "best_theta", "best_psi", "best_defocus",
                    "correlation_mean", "correlation_variance")}
            check(
                lib().lgb_match_finalize(
                    ctypes.byref(self.problem),
                    self.searched_projections,
                    _ptr(self.mip),
                    _ptr(self.best_index),
                    _ptr(self.corr_sum),
                    _ptr(self.corr_sq_sum),
                    _ptr(self.decode_euler if self.transpose else self.euler_angles),
                    _ptr(self.defocus_values),
                    _ptr(out["scaled_mip"]),
                    _ptr(out["best_phi"]),
                    _ptr(out["best_theta"]),
                    _ptr(out["best_psi"]),
                    _ptr(out["best_defocus"]),
                    _ptr(out["correlation_mean"]),
                    _ptr(out["correlation_variance"]),
                    s,
                ),
                "lgb_match_finalize",
            )
            res = {
                "mip": self.mip.clone(),
                "scaled_mip": out["scaled_mip"],
                "best_phi": out["best_phi"],
                "best_theta": out["best_theta"],
                "best_psi": out["best_psi"],
                "best_defocus": out["best_defocus"],
                "correlation_mean": out["correlation_mean"],
                "correlation_variance": out["correlation_variance"],
            }
            if (Hp, Wp) != (H, W):
                res = {k: v[:H, :W].contiguous() for k, v in res.items()}
            if self.transpose:
                res = {k: v.t().contiguous() for k, v in res.items()}
            if to_cpu:
                # page-locked destinations (torch's caching host allocator reuses
                # them across calls): the 8 maps go back as asynchronous copies
                # at full link speed, with one synchronisation
                host = {}
                for k, v in res.items():
                    h = torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
                    h.copy_(v, non_blocking=True)
                    host[k] = h
                torch.cuda.current_stream(dev).synchronize()
                res = host
        res["total_projections"] = self.total_projections
        res["total_orientations"] = self.problem.n_orientations
        res["total_defocus"] = self.problem.n_defocus
        return res


def core_match_template(
    image_dft: torch.Tensor,
    template_dft: torch.Tensor,
    ctf_filters: torch.Tensor,
    whitening_filter_template: torch.Tensor,
    defocus_values: torch.Tensor,
    pixel_values: torch.Tensor,
    euler_angles: torch.Tensor,
    device: torch.device | list[torch.device],
    orientation_batch_size: int = 1,
    num_cuda_streams: int = 1,
    backend: str = "streamed",
    mag_matrix: torch.Tensor | None = None,
) -> dict:
    """Whole-orientation 2DTM search; see leopard_em.backend.core_match_template.

    ``num_cuda_streams`` and ``backend`` are accepted for compatibility: both of
    the reference's backends compute the same correlograms, and here they map to
    the same fused kernel sequence on one stream.  Returns CPU tensors.
    """
    if backend not in ("streamed", "batched"):
        raise ValueError(f"backend must be 'streamed' or 'batched', got {backend!r}")
    if mag_matrix is not None:
        raise ValueError("anisotropic magnification (mag_matrix) is not supported by leopard_em_gb300")
    if num_cuda_streams > 1:
        warnings.warn(
            "num_cuda_streams is ignored: leopard_em_gb300 runs the search as one fused kernel "
            "sequence on the current CUDA stream",
            stacklevel=2,
        )
    # orientation batches replayed as CUDA graphs of ~128 orientations (same
    # results bit for bit; removes the per-kernel launch cost of small images)
    graph_batches = max(1, 128 // max(1, int(orientation_batch_size)))
    search = MatchTemplateSearch(
        image_dft,
        template_dft,
        ctf_filters,
        whitening_filter_template,
        defocus_values,
        pixel_values,
        euler_angles,
        device,
        orientation_batch_size,
        graph_batches=graph_batches,
    )
    search.run()
    return search.result(to_cpu=True)
