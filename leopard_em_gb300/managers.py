"""Manager-level API: ``MatchTemplateManager`` and ``RefineTemplateManager``.

Plain-Python mirrors (dataclasses, same field names and methods) of Leopard-EM's
pydantic managers and configs, backed by the GB300 kernels:

* ``DefocusSearchConfig`` / ``PixelSizeSearchConfig`` -- get_search_tensors
  (utils/search_utils.py:57-93; config/defocus_search.py:12-74);
* ``OrientationSearchConfig`` -- uniform SO(3) grid from psi/theta steps
  (config/orientation_search.py:22-170; the grid is this package's own
  uniform theta/phi/psi construction, an input to the search like the
  reference's torch-so3 grid);
* ``RefineOrientationConfig`` -- local offsets in [-coarse, +coarse] every fine
  step (config/orientation_search.py:205-278);
* ``OpticsGroup``, ``PreprocessingFilters``, ``ComputationalConfigMatch/Refine``;
* ``MatchTemplateResult.apply_valid_cropping`` (results/match_template_result.py:206-236);
* ``MatchTemplateManager.make_backend_core_function_kwargs`` /
  ``run_match_template`` (managers/match_template_manager.py:140-255, 327-358);
* ``RefineTemplateManager.run_refine_template`` over in-memory particle crops
  (managers/refine_template_manager.py:243-353, without the DataFrame-backed
  ParticleStack: crops and per-particle parameters are passed in directly).
File I/O (MRC, CSV) and YAML schema handling are not part of this package.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import torch

from . import grids
from . import preprocess as pp
from .backend import core_match_template, core_refine_template


def get_search_tensors(min_val: float, max_val: float, step_size: float, skip_enforce_zero: bool = False):
    """arange(min, max + step, step) with 0 inserted unless present (search_utils.py:57-93)."""
    vals = torch.arange(min_val, max_val + step_size, step_size, dtype=torch.float32)
    if abs(torch.min(torch.abs(vals))) > 1e-6 and not skip_enforce_zero:
        vals = torch.sort(torch.cat([vals, torch.tensor([0.0])]))[0]
    return vals


@dataclass
class DefocusSearchConfig:
    enabled: bool = True
    defocus_min: float = -1000.0
    defocus_max: float = 1000.0
    defocus_step: float = 200.0
    skip_enforce_zero: bool = False

    def __post_init__(self):
        if self.defocus_step <= 0:
            raise ValueError("defocus_step must be > 0")

    @property
    def defocus_values(self) -> torch.Tensor:
        if not self.enabled:
            return torch.tensor([0.0])
        if self.defocus_max < self.defocus_min:
            raise ValueError("Defocus search parameters result in no values to search over!")
        return get_search_tensors(self.defocus_min, self.defocus_max, self.defocus_step, self.skip_enforce_zero)


@dataclass
class PixelSizeSearchConfig:
    enabled: bool = False
    pixel_size_min: float = -0.05
    pixel_size_max: float = 0.05
    pixel_size_step: float = 0.01
    skip_enforce_zero: bool = False

    @property
    def pixel_size_values(self) -> torch.Tensor:
        if not self.enabled:
            return torch.tensor([0.0])
        return get_search_tensors(self.pixel_size_min, self.pixel_size_max, self.pixel_size_step,
                                  self.skip_enforce_zero)


@dataclass
class OrientationSearchConfig:
    psi_step: float = 1.5
    theta_step: float = 2.5

    @property
    def euler_angles(self) -> torch.Tensor:
        return grids.uniform_euler_grid(self.theta_step, self.psi_step)


@dataclass
class RefineOrientationConfig:
    enabled: bool = True
    psi_step_coarse: float = 1.5
    psi_step_fine: float = 0.1
    theta_step_coarse: float = 2.5
    theta_step_fine: float = 0.25

    @property
    def euler_angles_offsets(self) -> torch.Tensor:
        if not self.enabled:
            return torch.zeros((1, 3))
        return grids.local_euler_offsets(self.theta_step_coarse, self.theta_step_fine, self.psi_step_coarse,
                                         self.psi_step_fine)


@dataclass
class OpticsGroup:
    label: str = "default"
    pixel_size: float = 1.0
    voltage: float = 300.0
    spherical_aberration: float = 2.7
    amplitude_contrast_ratio: float = 0.07
    phase_shift: float = 0.0
    defocus_u: float = 10000.0
    defocus_v: float = 10000.0
    astigmatism_angle: float = 0.0
    ctf_B_factor: float = 0.0
    mag_matrix: Optional[list] = None

    @property
    def mag_matrix_tensor(self):
        if self.mag_matrix is None:
            return None
        m = self.mag_matrix
        return torch.tensor([[m[0], m[1]], [m[2], m[3]]], dtype=torch.float32)


@dataclass
class WhiteningFilterConfig:
    enabled: bool = True


@dataclass
class BandpassFilterConfig:
    """Raised-cosine band between low and high cutoffs (fractions of Nyquist
    spatial frequency 0.5); disabled -> all ones."""

    enabled: bool = False
    low_freq_cutoff: Optional[float] = None
    high_freq_cutoff: Optional[float] = None
    falloff: Optional[float] = None

    def calculate_bandpass_filter(self, output_shape, device=None) -> torch.Tensor:
        h, wc = output_shape
        if not self.enabled:
            return torch.ones((h, wc), dtype=torch.float32, device=device)
        ky, kx = pp.rfft_freq_grid((h, 2 * (wc - 1)), device=device)
        r = torch.sqrt(kx**2 + ky**2)
        lo = self.low_freq_cutoff or 0.0
        hi = self.high_freq_cutoff if self.high_freq_cutoff is not None else 1.0
        fo = self.falloff or 0.0
        f = torch.ones_like(r)
        if fo > 0:
            f = torch.where(r < lo, 0.5 * (1 + torch.cos(math.pi * torch.clamp((lo - r) / fo, 0, 1))), f)
            f = torch.where(r > hi, 0.5 * (1 + torch.cos(math.pi * torch.clamp((r - hi) / fo, 0, 1))), f)
        else:
            f = ((r >= lo) & (r <= hi)).to(r.dtype)
        return f.to(torch.float32)


@dataclass
class PreprocessingFilters:
    whitening_filter: WhiteningFilterConfig = field(default_factory=WhiteningFilterConfig)
    bandpass_filter: BandpassFilterConfig = field(default_factory=BandpassFilterConfig)

    def get_combined_filter(self, ref_img_rfft: torch.Tensor, output_shape) -> torch.Tensor:
        h, wc = output_shape
        dev = ref_img_rfft.device
        if self.whitening_filter.enabled:
            wf = pp.whitening_filter(ref_img_rfft, (h, 2 * (wc - 1)))
        else:
            wf = torch.ones((h, wc), dtype=torch.float32, device=dev)
        return wf * self.bandpass_filter.calculate_bandpass_filter(output_shape, device=dev)


@dataclass
class ComputationalConfigMatch:
    gpu_ids: object = 0
    num_cpus: int = 1
    backend: str = "streamed"

    @property
    def gpu_devices(self) -> list:
        ids = self.gpu_ids if isinstance(self.gpu_ids, list) else [self.gpu_ids]
        return [torch.device(f"cuda:{i}") if isinstance(i, int) else torch.device(i) for i in ids]


@dataclass
class ComputationalConfigRefine(ComputationalConfigMatch):
    pass


@dataclass
class MatchTemplateResult:
    mip: Optional[torch.Tensor] = None
    scaled_mip: Optional[torch.Tensor] = None
    correlation_average: Optional[torch.Tensor] = None
    correlation_variance: Optional[torch.Tensor] = None
    orientation_psi: Optional[torch.Tensor] = None
    orientation_theta: Optional[torch.Tensor] = None
    orientation_phi: Optional[torch.Tensor] = None
    relative_defocus: Optional[torch.Tensor] = None
    total_projections: int = 0
    total_orientations: int = 0
    total_defocus: int = 0
    allow_file_overwrite: bool = False
    mip_path: str = ""
    scaled_mip_path: str = ""
    correlation_average_path: str = ""
    correlation_variance_path: str = ""
    orientation_psi_path: str = ""
    orientation_theta_path: str = ""
    orientation_phi_path: str = ""
    relative_defocus_path: str = ""

    MAPS = ("mip", "scaled_mip", "correlation_average", "correlation_variance", "orientation_psi",
            "orientation_theta", "orientation_phi", "relative_defocus")

    def export_results(self) -> None:
        """Write the eight maps to their MRC paths (match_template_result.py:308-340)."""
        from .mrc import write_mrc

        for name in self.MAPS:
            path = getattr(self, f"{name}_path")
            if not path:
                raise ValueError(f"{name}_path is not set")
            write_mrc(path, getattr(self, name), overwrite=self.allow_file_overwrite)

    def load_tensors_from_paths(self) -> None:
        """Read the eight maps back from their MRC paths (match_template_result.py:238-250)."""
        from .mrc import read_mrc

        for name in self.MAPS:
            setattr(self, name, torch.from_numpy(read_mrc(getattr(self, f"{name}_path"))).to(torch.float32))

    def apply_valid_cropping(self, template_shape) -> None:
        """Crop every map to (H - h + 1, W - w + 1) (match_template_result.py:206-236)."""
        img_h, img_w = self.mip.shape
        h, w = template_shape
        sl = (slice(img_h - h + 1), slice(img_w - w + 1))
        for name in ("mip", "scaled_mip", "correlation_average", "correlation_variance", "orientation_psi",
                     "orientation_theta", "orientation_phi", "relative_defocus"):
            setattr(self, name, getattr(self, name)[sl])

    match_template_peaks: Optional["MatchTemplatePeaks"] = None

    def locate_peaks(self, **kwargs) -> "MatchTemplatePeaks":
        """Peak positions and per-peak statistics from the held maps
        (match_template_result.py:252-288), with the z-score peak picking on the
        device (``peaks.extract_peaks_and_statistics_zscore``; keyword
        arguments: false_positives, z_score_cutoff, mask_radius, device)."""
        from .peaks import extract_peaks_and_statistics_zscore

        self.match_template_peaks = extract_peaks_and_statistics_zscore(
            mip=self.mip,
            scaled_mip=self.scaled_mip,
            best_psi=self.orientation_psi,
            best_theta=self.orientation_theta,
            best_phi=self.orientation_phi,
            best_defocus=self.relative_defocus,
            correlation_average=self.correlation_average,
            correlation_variance=self.correlation_variance,
            total_correlation_positions=self.total_projections,
            **kwargs,
        )
        return self.match_template_peaks

    def peaks_to_dict(self) -> dict:
        """The located peaks as a dictionary (match_template_result.py:290-295)."""
        if self.match_template_peaks is None:
            self.locate_peaks()
        return self.match_template_peaks._asdict()


@dataclass
class MatchTemplateManager:
    micrograph: torch.Tensor
    template_volume: torch.Tensor
    optics_group: OpticsGroup = field(default_factory=OpticsGroup)
    defocus_search_config: DefocusSearchConfig = field(default_factory=DefocusSearchConfig)
    orientation_search_config: OrientationSearchConfig = field(default_factory=OrientationSearchConfig)
    preprocessing_filters: PreprocessingFilters = field(default_factory=PreprocessingFilters)
    match_template_result: MatchTemplateResult = field(default_factory=MatchTemplateResult)
    computational_config: ComputationalConfigMatch = field(default_factory=ComputationalConfigMatch)
    micrograph_path: str = ""
    template_volume_path: str = ""

    def make_backend_core_function_kwargs(self, preprocess_device=None) -> dict:
        """Backend inputs from held parameters (match_template_manager.py:140-218).

        ``preprocess_device`` (e.g. "cuda:0") runs the image rfft, the
        whitening and bandpass filters, the CTF stack and the template rfft
        there instead of on the host; the returned tensors live on it."""
        dev = torch.device(preprocess_device) if preprocess_device is not None else torch.device("cpu")
        image = torch.as_tensor(self.micrograph, dtype=torch.float32).to(dev)
        template = torch.as_tensor(self.template_volume, dtype=torch.float32).to(dev)
        image_dft = torch.fft.rfftn(image)
        image_dft[0, 0] = 0 + 0j
        bandpass = self.preprocessing_filters.bandpass_filter.calculate_bandpass_filter(image_dft.shape, device=dev)
        cum_img = self.preprocessing_filters.get_combined_filter(image_dft, image_dft.shape)
        cum_tmp = self.preprocessing_filters.get_combined_filter(
            image_dft, (template.shape[-2], template.shape[-1] // 2 + 1))
        image_pre = pp.preprocess_image(image_dft, cum_img, bandpass, tuple(image.shape[-2:]),
                                        tuple(image.shape[-2:]))
        defocus_values = self.defocus_search_config.defocus_values
        pixel_size_offsets = torch.tensor([0.0], dtype=torch.float32)
        og = self.optics_group
        ctf = pp.ctf_filter_stack(template.shape[0], og.defocus_u, og.defocus_v, defocus_values, pixel_size_offsets,
                                  astigmatism_angle=og.astigmatism_angle, voltage=og.voltage,
                                  spherical_aberration=og.spherical_aberration,
                                  amplitude_contrast=og.amplitude_contrast_ratio, phase_shift=og.phase_shift,
                                  pixel_size=og.pixel_size, b_factor=og.ctf_B_factor, device=dev)
        return {
            "image_dft": image_pre.to(torch.complex64),
            "template_dft": pp.volume_to_rfft_fourier_slice(template).to(torch.complex64),
            "ctf_filters": ctf,
            "whitening_filter_template": cum_tmp,
            "euler_angles": self.orientation_search_config.euler_angles.to(torch.float32),
            "defocus_values": defocus_values,
            "pixel_values": pixel_size_offsets,
            "device": self.computational_config.gpu_devices,
            "mag_matrix": og.mag_matrix_tensor,
        }

    def run_match_template(self, orientation_batch_size: int = 16, do_result_export: bool = True,
                           do_valid_cropping: bool = True) -> None:
        """Run the search and populate ``match_template_result`` (:220-255, :327-358).
        Pre-processing runs on the search's GPU."""
        kw = self.make_backend_core_function_kwargs(preprocess_device=self.computational_config.gpu_devices[0])
        res = core_match_template(**kw, orientation_batch_size=orientation_batch_size,
                                  num_cuda_streams=self.computational_config.num_cpus,
                                  backend=self.computational_config.backend)
        r = self.match_template_result
        r.mip, r.scaled_mip = res["mip"], res["scaled_mip"]
        r.correlation_average, r.correlation_variance = res["correlation_mean"], res["correlation_variance"]
        r.orientation_psi, r.orientation_theta, r.orientation_phi = res["best_psi"], res["best_theta"], res["best_phi"]
        r.relative_defocus = res["best_defocus"]
        r.total_projections = res["total_projections"]
        r.total_orientations = res["total_orientations"]
        r.total_defocus = res["total_defocus"]
        if do_valid_cropping:
            nx = self.template_volume.shape[-1]
            r.apply_valid_cropping((nx, nx))
        if do_result_export:
            r.export_results()


@dataclass
class RefineTemplateManager:
    """Refinement of particles given as in-memory crops (no ParticleStack).

    ``particle_images``: (N, H, W) real crops; per-particle ``euler_angles``
    (N, 3), ``defocus_u/v/angle`` (N,); ``corr_mean`` / ``corr_std``
    (N, H-d+1, W-d+1) from the search (default 0 / 1).
    """

    particle_images: torch.Tensor
    template_volume: torch.Tensor
    euler_angles: torch.Tensor
    defocus_u: torch.Tensor
    defocus_v: torch.Tensor
    defocus_angle: torch.Tensor
    optics_group: OpticsGroup = field(default_factory=OpticsGroup)
    defocus_refinement_config: DefocusSearchConfig = field(default_factory=lambda: DefocusSearchConfig(
        defocus_min=-100.0, defocus_max=100.0, defocus_step=20.0))
    pixel_size_refinement_config: PixelSizeSearchConfig = field(default_factory=PixelSizeSearchConfig)
    orientation_refinement_config: RefineOrientationConfig = field(default_factory=RefineOrientationConfig)
    preprocessing_filters: PreprocessingFilters = field(default_factory=PreprocessingFilters)
    computational_config: ComputationalConfigRefine = field(default_factory=ComputationalConfigRefine)
    corr_mean: Optional[torch.Tensor] = None
    corr_std: Optional[torch.Tensor] = None

    def make_backend_core_function_kwargs(self) -> dict:
        imgs = torch.as_tensor(self.particle_images, dtype=torch.float32)
        n, H, W = imgs.shape
        template = torch.as_tensor(self.template_volume, dtype=torch.float32)
        d = template.shape[-1]
        dfts = torch.fft.rfftn(imgs, dim=(-2, -1))
        dfts[:, 0, 0] = 0 + 0j
        pre, pfs = [], []
        for i in range(n):
            bp = self.preprocessing_filters.bandpass_filter.calculate_bandpass_filter(dfts[i].shape)
            cf = self.preprocessing_filters.get_combined_filter(dfts[i], dfts[i].shape)
            pre.append(pp.preprocess_image(dfts[i], cf, bp, (H, W), (H, W)))
            pfs.append(self.preprocessing_filters.get_combined_filter(dfts[i], (d, d // 2 + 1)))
        crop = (n, H - d + 1, W - d + 1)
        og = self.optics_group
        return {
            "particle_stack_dft": torch.stack(pre).to(torch.complex64),
            "template_dft": pp.volume_to_rfft_fourier_slice(template).to(torch.complex64),
            "euler_angles": torch.as_tensor(self.euler_angles, dtype=torch.float32),
            "euler_angle_offsets": self.orientation_refinement_config.euler_angles_offsets,
            "defocus_offsets": self.defocus_refinement_config.defocus_values,
            "defocus_u": torch.as_tensor(self.defocus_u, dtype=torch.float32),
            "defocus_v": torch.as_tensor(self.defocus_v, dtype=torch.float32),
            "defocus_angle": torch.as_tensor(self.defocus_angle, dtype=torch.float32),
            "pixel_size_offsets": self.pixel_size_refinement_config.pixel_size_values,
            "corr_mean": self.corr_mean if self.corr_mean is not None else torch.zeros(crop),
            "corr_std": self.corr_std if self.corr_std is not None else torch.ones(crop),
            "ctf_kwargs": dict(voltage=og.voltage, spherical_aberration=og.spherical_aberration,
                               amplitude_contrast_ratio=og.amplitude_contrast_ratio, ctf_B_factor=og.ctf_B_factor,
                               phase_shift=og.phase_shift, pixel_size=og.pixel_size, template_shape=(d, d),
                               even_zernikes=None, odd_zernikes=None, mag_matrix=None),
            "projective_filters": torch.stack(pfs),
            "device": self.computational_config.gpu_devices,
        }

    def run_refine_template(self, orientation_batch_size: int = 64) -> dict:
        kw = self.make_backend_core_function_kwargs()
        return core_refine_template(**kw, batch_size=orientation_batch_size,
                                    num_cuda_streams=self.computational_config.num_cpus)
