"""Manager-level API: ``MatchTemplateManager`` and ``RefineTemplateManager``.

Validated configuration models with the reference's class names, field names,
defaults, ranges and YAML / JSON round trips (``config_models.ConfigModel``;
the reference's models are pydantic, ``pydantic_models/``), backed by the
GB300 kernels:

* ``DefocusSearchConfig`` / ``PixelSizeSearchConfig`` -- get_search_tensors
  (utils/search_utils.py:57-93; config/defocus_search.py:12-74,
  config/pixel_size_search.py:12-72);
* ``OrientationSearchConfig`` / ``MultipleOrientationConfig`` -- the uniform
  SO(3) grid over symmetry or explicit angle ranges
  (config/orientation_search.py:22-203; ``grids.uniform_euler_angles``);
* ``RefineOrientationConfig`` -- the local refinement grid
  (config/orientation_search.py:205-278; ``grids.local_high_resolution_angles``);
* ``OpticsGroup`` (data_structures/optics_group.py:12-113),
  ``MovieConfig`` (config/movie_config.py), the correlation filters and
  ``PreprocessingFilters`` (config/correlation_filters.py:16-410),
  ``ComputationalConfigMatch/Refine`` (config/computational_config.py);
* ``MatchTemplateResult`` (results/match_template_result.py:48-337);
* ``MatchTemplateManager`` (managers/match_template_manager.py:92-358) and
  ``RefineTemplateManager`` (managers/refine_template_manager.py:32-353) over
  a ``ParticleStack`` (``particle_stack.py``).
"""

from __future__ import annotations

import os
import re
from typing import Any, ClassVar, Literal, Optional, Union

import torch

from . import grids
from . import preprocess as pp
from .backend import core_match_template, core_refine_template
from .config_models import ConfigModel, Field, ValidationError
from .particle_stack import ParticleStack


def get_search_tensors(min_val: float, max_val: float, step_size: float, skip_enforce_zero: bool = False):
    """arange(min, max + step, step) with 0 inserted unless present (search_utils.py:57-93)."""
    vals = torch.arange(min_val, max_val + step_size, step_size, dtype=torch.float32)
    if abs(torch.min(torch.abs(vals))) > 1e-6 and not skip_enforce_zero:
        vals = torch.sort(torch.cat([vals, torch.tensor([0.0])]))[0]
    return vals


def load_mrc_image(path) -> torch.Tensor:
    """2-D float32 image from an MRC file (utils/data_io.py load_mrc_image)."""
    from .mrc import read_mrc

    arr = read_mrc(path)
    if arr.ndim == 3 and arr.shape[0] == 1:
        arr = arr[0]
    if arr.ndim != 2:
        raise ValueError(f"'{path}' does not hold a 2-D image (shape {arr.shape})")
    return torch.from_numpy(arr.astype("float32"))


def load_mrc_volume(path) -> torch.Tensor:
    """3-D float32 volume from an MRC file (utils/data_io.py load_mrc_volume)."""
    from .mrc import read_mrc

    arr = read_mrc(path)
    if arr.ndim != 3:
        raise ValueError(f"'{path}' does not hold a 3-D volume (shape {arr.shape})")
    return torch.from_numpy(arr.astype("float32"))


# ---------------------------------------------------------------------------
# Search ranges
# ---------------------------------------------------------------------------


class DefocusSearchConfig(ConfigModel):
    enabled: bool = True
    defocus_min: float = -1000.0
    defocus_max: float = 1000.0
    defocus_step: float = Field(200.0, gt=0.0)
    skip_enforce_zero: bool = False

    @property
    def defocus_values(self) -> torch.Tensor:
        if not self.enabled:
            return torch.tensor([0.0])
        if self.defocus_max < self.defocus_min:
            raise ValueError("Defocus search parameters result in no values to search over!")
        return get_search_tensors(self.defocus_min, self.defocus_max, self.defocus_step, self.skip_enforce_zero)


class PixelSizeSearchConfig(ConfigModel):
    enabled: bool = False
    pixel_size_min: float = 0.0
    pixel_size_max: float = 0.0
    pixel_size_step: float = Field(0.0, gt=0.0)
    skip_enforce_zero: bool = False

    @property
    def pixel_size_values(self) -> torch.Tensor:
        if not self.enabled:
            return torch.tensor([0.0])
        if self.pixel_size_max < self.pixel_size_min:
            raise ValueError("Pixel size search parameters result in no values to search over!")
        return get_search_tensors(self.pixel_size_min, self.pixel_size_max, self.pixel_size_step,
                                  self.skip_enforce_zero)


class OrientationSearchConfig(ConfigModel):
    """Whole-orientation grid: either a symmetry group (the default "C1") or
    all six angle bounds, never both (orientation_search.py:84-124)."""

    psi_step: float = Field(1.5, ge=0.0)
    theta_step: float = Field(2.5, ge=0.0)
    phi_min: Optional[float] = None
    phi_max: Optional[float] = None
    theta_min: Optional[float] = None
    theta_max: Optional[float] = None
    psi_min: Optional[float] = None
    psi_max: Optional[float] = None
    base_grid_method: Literal["uniform", "healpix", "cartesian"] = "uniform"
    symmetry: Optional[str] = "C1"

    _ANGLES: ClassVar = ("phi_min", "phi_max", "theta_min", "theta_max", "psi_min", "psi_max")

    def validate(self) -> None:
        all_none = all(getattr(self, k) is None for k in self._ANGLES)
        if not self.symmetry and all_none:
            raise ValidationError("Either a symmetry group must be provided, or all angle ranges must not be None. "
                                  "Both symmetry and angle ranges were set to None.")
        if self.symmetry and not all_none:
            raise ValidationError("Symmetry group is provided, but angle ranges are also set. "
                                  "Please set all angle ranges to None when using symmetry.")
        if self.symmetry and not re.match(r"([A-Za-z]+)(\d*)$", self.symmetry):
            raise ValidationError(f"Invalid symmetry format: {self.symmetry}")

    @property
    def euler_angles(self) -> torch.Tensor:
        if self.base_grid_method == "healpix":
            raise ValueError("base_grid_method 'healpix' is not supported by leopard_em_gb300 (uniform, cartesian)")
        periodic = None
        if self.symmetry is not None:
            periodic = True
            m = re.match(r"([A-Za-z]+)(\d*)", self.symmetry)
            order = int(m.group(2)) if m.group(2) else 1
            phi_min, phi_max, theta_min, theta_max, psi_min, psi_max = grids.symmetry_ranges(m.group(1), order)
        else:
            phi_min = self.phi_min if self.phi_min is not None else 0.0
            phi_max = self.phi_max if self.phi_max is not None else 360.0
            theta_min = self.theta_min if self.theta_min is not None else 0.0
            theta_max = self.theta_max if self.theta_max is not None else 180.0
            psi_min = self.psi_min if self.psi_min is not None else 0.0
            psi_max = self.psi_max if self.psi_max is not None else 360.0
        return grids.uniform_euler_angles(psi_step=self.psi_step, theta_step=self.theta_step, phi_min=phi_min,
                                          phi_max=phi_max, theta_min=theta_min, theta_max=theta_max,
                                          psi_min=psi_min, psi_max=psi_max, base_grid_method=self.base_grid_method,
                                          psi_periodic=periodic)


class MultipleOrientationConfig(ConfigModel):
    """Concatenated grids of several ``OrientationSearchConfig`` (:172-203)."""

    orientation_configs: list[OrientationSearchConfig]

    @property
    def euler_angles(self) -> torch.Tensor:
        return torch.cat([c.euler_angles for c in self.orientation_configs], dim=0)


class RefineOrientationConfig(ConfigModel):
    enabled: bool = True
    phi_step_coarse: float = Field(2.5, ge=0.0)
    phi_step_fine: float = Field(0.25, ge=0.0)
    theta_step_coarse: float = Field(2.5, ge=0.0)
    theta_step_fine: float = Field(0.25, ge=0.0)
    psi_step_coarse: float = Field(1.5, ge=0.0)
    psi_step_fine: float = Field(0.1, ge=0.0)
    base_grid_method: Literal["uniform", "healpix", "basic"] = "uniform"

    @property
    def euler_angles_offsets(self) -> torch.Tensor:
        if not self.enabled:
            return torch.zeros((1, 3))
        if self.base_grid_method == "healpix":
            raise ValueError("base_grid_method 'healpix' is not supported by leopard_em_gb300 (uniform, basic)")
        return grids.local_high_resolution_angles(
            coarse_phi_step=self.phi_step_coarse, coarse_theta_step=self.theta_step_coarse,
            coarse_psi_step=self.psi_step_coarse, fine_phi_step=self.phi_step_fine,
            fine_theta_step=self.theta_step_fine, fine_psi_step=self.psi_step_fine,
            base_grid_method=self.base_grid_method)


# ---------------------------------------------------------------------------
# Optics, movies, filters, devices
# ---------------------------------------------------------------------------


class OpticsGroup(ConfigModel):
    label: str
    pixel_size: float = Field(ge=0.0)
    voltage: float = Field(ge=0.0)
    spherical_aberration: float = Field(2.7, ge=0.0)
    amplitude_contrast_ratio: float = Field(0.07, ge=0.0, le=1.0)
    phase_shift: float = 0.0
    defocus_u: float
    defocus_v: float
    astigmatism_angle: float
    ctf_B_factor: float = Field(0.0, ge=0.0)
    chromatic_aberration: Optional[float] = Field(0.0, ge=0.0)
    mtf_reference: Optional[str] = None
    mtf_values: Optional[list[float]] = None
    beam_tilt_x: Optional[float] = None
    beam_tilt_y: Optional[float] = None
    odd_zernikes: Optional[dict[str, float]] = None
    even_zernikes: Optional[dict[str, float]] = None
    mag_matrix: Optional[list[float]] = Field(None, min_length=4, max_length=4)

    @property
    def mag_matrix_tensor(self):
        if self.mag_matrix is None:
            return None
        m = self.mag_matrix
        return torch.tensor([[m[0], m[1]], [m[2], m[3]]], dtype=torch.float32)


class MovieConfig(ConfigModel):
    """Movie-frame particle extraction (config/movie_config.py).  Only the
    disabled form is supported: per-frame extraction with deformation fields
    is not part of this package."""

    enabled: bool = False
    movie_path: str = ""
    deformation_field_path: str = ""
    particle_shifts_path: str = ""
    pre_exposure: float = 0.0
    fluence_per_frame: float = 1.0

    @property
    def movie(self):
        if not self.enabled:
            return None
        return load_mrc_volume(self.movie_path)


class WhiteningFilterConfig(ConfigModel):
    enabled: bool = True
    num_freq_bins: Optional[int] = None
    max_freq: Optional[float] = 0.5
    do_power_spectrum: Optional[bool] = True

    def calculate_whitening_filter(self, ref_img_rfft: torch.Tensor, output_shape=None) -> torch.Tensor:
        if output_shape is None:
            output_shape = tuple(ref_img_rfft.shape)
        if not self.enabled:
            return torch.ones(tuple(output_shape), dtype=torch.float32, device=ref_img_rfft.device)
        h, wc = output_shape[-2], output_shape[-1]
        return pp.whitening_filter(ref_img_rfft, (h, 2 * (wc - 1)), num_bins=self.num_freq_bins,
                                   max_freq=self.max_freq, do_power_spectrum=bool(self.do_power_spectrum))


class PhaseRandomizationFilterConfig(ConfigModel):
    enabled: bool = False
    cuton: Optional[float] = Field(None, ge=0.0)

    def calculate_phase_randomization_filter(self, ref_img_rfft: torch.Tensor) -> torch.Tensor:
        if not self.enabled:
            return torch.ones(tuple(ref_img_rfft.shape), dtype=torch.float32, device=ref_img_rfft.device)
        raise ValueError("phase randomization is not supported by leopard_em_gb300")


class BandpassFilterConfig(ConfigModel):
    """Raised-cosine band between low and high cutoffs (fractions of the
    sampling frequency; Nyquist = 0.5); disabled -> all ones."""

    enabled: bool = False
    low_freq_cutoff: Optional[float] = Field(None, ge=0.0)
    high_freq_cutoff: Optional[float] = Field(None, ge=0.0)
    falloff: Optional[float] = Field(None, ge=0.0)

    @classmethod
    def from_spatial_resolution(cls, low_resolution: float, high_resolution: float, pixel_size: float, **kwargs):
        return cls(low_freq_cutoff=pixel_size / low_resolution, high_freq_cutoff=pixel_size / high_resolution,
                   **kwargs)

    def calculate_bandpass_filter(self, output_shape, device=None) -> torch.Tensor:
        h, wc = output_shape[-2], output_shape[-1]
        if not self.enabled:
            return torch.ones((h, wc), dtype=torch.float32, device=device)
        return pp.bandpass_filter((h, 2 * (wc - 1)), self.low_freq_cutoff or 0.0,
                                  1.0 if self.high_freq_cutoff is None else self.high_freq_cutoff,
                                  self.falloff or 0.0, device=device)


class ArbitraryCurveFilterConfig(ConfigModel):
    enabled: bool = False
    frequencies: Optional[list[float]] = None
    amplitudes: Optional[list[float]] = None

    def calculate_arbitrary_curve_filter(self, output_shape, device=None) -> torch.Tensor:
        h, wc = output_shape[-2], output_shape[-1]
        if not self.enabled:
            return torch.ones((h, wc), dtype=torch.float32, device=device)
        if self.frequencies is None or self.amplitudes is None:
            raise ValueError("When enabled, both 'frequencies' and 'amplitudes' must be provided.")
        return pp.radial_curve_filter((h, 2 * (wc - 1)), self.frequencies, self.amplitudes, device=device)


class PreprocessingFilters(ConfigModel):
    whitening_filter: WhiteningFilterConfig = WhiteningFilterConfig()
    bandpass_filter: BandpassFilterConfig = BandpassFilterConfig()
    phase_randomization_filter: PhaseRandomizationFilterConfig = PhaseRandomizationFilterConfig()
    arbitrary_curve_filter: ArbitraryCurveFilterConfig = ArbitraryCurveFilterConfig()

    def get_combined_filter(self, ref_img_rfft: torch.Tensor, output_shape) -> torch.Tensor:
        """whitening x bandpass x arbitrary curve (correlation_filters.py:366-410)."""
        dev = ref_img_rfft.device
        wf = self.whitening_filter.calculate_whitening_filter(ref_img_rfft, output_shape).to(dev)
        bp = self.bandpass_filter.calculate_bandpass_filter(output_shape, device=dev)
        ac = self.arbitrary_curve_filter.calculate_arbitrary_curve_filter(output_shape, device=dev)
        return wf * bp * ac


class ComputationalConfigMatch(ConfigModel):
    gpu_ids: Optional[Union[str, int, list[int], list[str]]] = [0]
    num_cpus: int = Field(1, ge=1)
    backend: Literal["streamed", "batched"] = "streamed"

    def validate(self) -> None:
        if isinstance(self.gpu_ids, int) and self.gpu_ids < 0:
            raise ValidationError("gpu_ids: Input should be greater than or equal to 0")
        if isinstance(self.gpu_ids, list):
            if not self.gpu_ids:
                raise ValidationError("gpu_ids: should have at least 1 item")
            if any(isinstance(i, int) and i < 0 for i in self.gpu_ids):
                raise ValidationError("gpu_ids: Input should be greater than or equal to 0")

    @property
    def gpu_devices(self) -> list:
        if self.gpu_ids == "all":
            if not torch.cuda.is_available():
                raise ValueError("No CUDA devices available.")
            return [torch.device(f"cuda:{i}") for i in range(torch.cuda.device_count())]
        if self.gpu_ids == "cpu":
            return [torch.device("cpu")]
        ids = self.gpu_ids if isinstance(self.gpu_ids, list) else [self.gpu_ids]
        return [torch.device(f"cuda:{i}") if isinstance(i, int) else torch.device(i) for i in ids]


class ComputationalConfigRefine(ComputationalConfigMatch):
    backend: Literal["streamed", "batched"] = "batched"


# ---------------------------------------------------------------------------
# Results
# ---------------------------------------------------------------------------


def check_file_path_and_permissions(path: str, allow_overwrite: bool) -> None:
    """Create the parent folder, require write access, and refuse an existing
    file unless overwriting is allowed (match_template_result.py:24-45)."""
    directory = os.path.dirname(path)
    if directory and not os.path.exists(directory):
        os.makedirs(directory, exist_ok=True)
    if directory and not os.access(directory, os.W_OK):
        raise ValueError(f"Directory '{directory}' does not permit writing. Will be unable to write results to "
                         f"'{path}'.")
    if not allow_overwrite and os.path.exists(path):
        raise ValueError(f"File '{path}' already exists, but 'allow_file_overwrite' is False.")


class MatchTemplateResult(ConfigModel):
    allow_file_overwrite: bool = False
    mip_path: str
    scaled_mip_path: str
    correlation_average_path: str
    correlation_variance_path: str
    orientation_psi_path: str
    orientation_theta_path: str
    orientation_phi_path: str
    relative_defocus_path: str
    total_projections: int = 0
    total_orientations: int = 0
    total_defocus: int = 0
    match_template_peaks: Any = Field(None, exclude=True)
    mip: Any = Field(None, exclude=True)
    scaled_mip: Any = Field(None, exclude=True)
    correlation_average: Any = Field(None, exclude=True)
    correlation_variance: Any = Field(None, exclude=True)
    orientation_psi: Any = Field(None, exclude=True)
    orientation_theta: Any = Field(None, exclude=True)
    orientation_phi: Any = Field(None, exclude=True)
    relative_defocus: Any = Field(None, exclude=True)

    MAPS: ClassVar = ("mip", "scaled_mip", "correlation_average", "correlation_variance", "orientation_psi",
                      "orientation_theta", "orientation_phi", "relative_defocus")

    def validate(self) -> None:
        for name in self.MAPS:
            check_file_path_and_permissions(getattr(self, f"{name}_path"), self.allow_file_overwrite)

    def export_results(self) -> None:
        """Write the eight maps to their MRC paths (match_template_result.py:308-337)."""
        from .mrc import write_mrc

        for name in self.MAPS:
            write_mrc(getattr(self, f"{name}_path"), getattr(self, name), overwrite=self.allow_file_overwrite)

    def load_tensors_from_paths(self) -> None:
        """Read the eight maps back from their MRC paths (match_template_result.py:238-250)."""
        for name in self.MAPS:
            setattr(self, name, load_mrc_image(getattr(self, f"{name}_path")))

    def apply_valid_cropping(self, template_shape) -> None:
        """Crop every map to (H - h + 1, W - w + 1) (match_template_result.py:206-236)."""
        img_h, img_w = self.mip.shape
        h, w = template_shape
        sl = (slice(img_h - h + 1), slice(img_w - w + 1))
        for name in self.MAPS:
            setattr(self, name, getattr(self, name)[sl])

    def locate_peaks(self, **kwargs):
        """Peak positions and per-peak statistics from the held maps
        (match_template_result.py:252-288), with the z-score peak picking on
        the device (``peaks.extract_peaks_and_statistics_zscore``; keyword
        arguments: false_positives, z_score_cutoff, mask_radius, device)."""
        from .peaks import extract_peaks_and_statistics_zscore

        self.match_template_peaks = extract_peaks_and_statistics_zscore(
            mip=self.mip, scaled_mip=self.scaled_mip, best_psi=self.orientation_psi,
            best_theta=self.orientation_theta, best_phi=self.orientation_phi, best_defocus=self.relative_defocus,
            correlation_average=self.correlation_average, correlation_variance=self.correlation_variance,
            total_correlation_positions=self.total_projections, **kwargs)
        return self.match_template_peaks

    def peaks_to_dict(self) -> dict:
        """The located peaks as a dictionary (match_template_result.py:290-295)."""
        if self.match_template_peaks is None:
            self.locate_peaks()
        return self.match_template_peaks._asdict()


# ---------------------------------------------------------------------------
# Managers
# ---------------------------------------------------------------------------


def calculate_ctf_filter_stack(template_shape, optics_group: OpticsGroup, defocus_offsets: torch.Tensor,
                               pixel_size_offsets: torch.Tensor, device=None) -> torch.Tensor:
    """(C, D, h, h//2+1) CTF stack of an optics group (utils/ctf_utils.py:19-116)."""
    og = optics_group
    if og.even_zernikes or og.odd_zernikes:
        raise ValueError("Zernike aberration terms are not supported by leopard_em_gb300")
    return pp.ctf_filter_stack(template_shape[0], og.defocus_u, og.defocus_v, defocus_offsets, pixel_size_offsets,
                               astigmatism_angle=og.astigmatism_angle, voltage=og.voltage,
                               spherical_aberration=og.spherical_aberration,
                               amplitude_contrast=og.amplitude_contrast_ratio, phase_shift=og.phase_shift,
                               pixel_size=og.pixel_size, b_factor=og.ctf_B_factor, device=device)


class MatchTemplateManager(ConfigModel):
    """Whole-orientation search of one micrograph (match_template_manager.py:92-358)."""

    micrograph_path: str
    template_volume_path: str
    optics_group: OpticsGroup
    defocus_search_config: DefocusSearchConfig
    orientation_search_config: Union[OrientationSearchConfig, MultipleOrientationConfig]
    preprocessing_filters: PreprocessingFilters
    match_template_result: MatchTemplateResult
    computational_config: ComputationalConfigMatch
    micrograph: Any = Field(None, exclude=True)
    template_volume: Any = Field(None, exclude=True)

    def __init__(self, preload_mrc_files: bool = False, **data: Any):
        super().__init__(**data)
        if preload_mrc_files:
            self.micrograph = load_mrc_image(self.micrograph_path)
            self.template_volume = load_mrc_volume(self.template_volume_path)

    def validate(self) -> None:
        if not os.path.exists(self.micrograph_path):
            raise ValidationError(f"File '{self.micrograph_path}' for micrograph does not exist.")
        if not os.path.exists(self.template_volume_path):
            raise ValidationError(f"File '{self.template_volume_path}' for template volume does not exist.")

    def make_backend_core_function_kwargs(self, preprocess_device=None) -> dict:
        """Backend inputs from held parameters (match_template_manager.py:140-218).

        ``preprocess_device`` (e.g. "cuda:0") runs the image rfft, the
        whitening and bandpass filters, the CTF stack and the template rfft
        there instead of on the host; the returned tensors live on it."""
        if self.micrograph is None:
            self.micrograph = load_mrc_image(self.micrograph_path)
        if self.template_volume is None:
            self.template_volume = load_mrc_volume(self.template_volume_path)
        dev = torch.device(preprocess_device) if preprocess_device is not None else torch.device("cpu")
        image = torch.as_tensor(self.micrograph, dtype=torch.float32).to(dev)
        template = torch.as_tensor(self.template_volume, dtype=torch.float32).to(dev)
        image_dft = torch.fft.rfftn(image)
        image_dft[0, 0] = 0 + 0j
        pf = self.preprocessing_filters
        bandpass = pf.bandpass_filter.calculate_bandpass_filter(image_dft.shape, device=dev)
        cum_img = pf.get_combined_filter(image_dft, tuple(image_dft.shape))
        cum_tmp = pf.get_combined_filter(image_dft, (template.shape[-2], template.shape[-1] // 2 + 1))
        image_pre = pp.preprocess_image(image_dft, cum_img, bandpass, tuple(image.shape[-2:]),
                                        tuple(image.shape[-2:]))
        defocus_values = self.defocus_search_config.defocus_values
        pixel_size_offsets = torch.tensor([0.0], dtype=torch.float32)
        ctf = calculate_ctf_filter_stack((template.shape[0], template.shape[0]), self.optics_group, defocus_values,
                                         pixel_size_offsets, device=dev)
        return {
            "image_dft": image_pre.to(torch.complex64),
            "template_dft": pp.volume_to_rfft_fourier_slice(template).to(torch.complex64),
            "ctf_filters": ctf,
            "whitening_filter_template": cum_tmp,
            "euler_angles": self.orientation_search_config.euler_angles.to(torch.float32),
            "defocus_values": defocus_values,
            "pixel_values": pixel_size_offsets,
            "device": self.computational_config.gpu_devices,
            "mag_matrix": self.optics_group.mag_matrix_tensor,
        }

    def run_match_template(self, orientation_batch_size: int = 16, do_result_export: bool = True,
                           do_valid_cropping: bool = True) -> None:
        """Run the search and populate ``match_template_result`` (:220-255, :327-358).
        Pre-processing runs on the search's GPU."""
        kw = self.make_backend_core_function_kwargs(preprocess_device=self.computational_config.gpu_devices[0])
        res = core_match_template(**kw, orientation_batch_size=orientation_batch_size,
                                  num_cuda_streams=self.computational_config.num_cpus,
                                  backend=self.computational_config.backend)
        self._populate_match_template_result(res, do_result_export, do_valid_cropping)

    def _populate_match_template_result(self, res: dict, do_result_export: bool = True,
                                        do_valid_cropping: bool = True) -> None:
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

    def save_config(self, path: str, mode: Literal["yaml", "json"] = "yaml") -> None:
        if mode == "yaml":
            self.to_yaml(path)
        elif mode == "json":
            self.to_json(path)
        else:
            raise ValueError(f"Invalid serialization mode '{mode}'.")


class RefineTemplateManager(ConfigModel):
    """Local refinement of the particles of a ``ParticleStack``
    (refine_template_manager.py:32-353)."""

    template_volume_path: str
    particle_stack: ParticleStack
    defocus_refinement_config: DefocusSearchConfig
    pixel_size_refinement_config: PixelSizeSearchConfig
    orientation_refinement_config: RefineOrientationConfig
    preprocessing_filters: PreprocessingFilters
    computational_config: ComputationalConfigRefine
    movie_config: MovieConfig = MovieConfig()
    apply_global_filtering: bool = True
    template_volume: Any = Field(None, exclude=True)

    def __init__(self, skip_mrc_preloads: bool = False, **data: Any):
        super().__init__(**data)
        if not skip_mrc_preloads:
            self.template_volume = load_mrc_volume(self.template_volume_path)

    def make_backend_core_function_kwargs(self, prefer_refined_angles: bool = True) -> dict:
        """Backend inputs (refine_template_manager.py:93-168 and
        utils/backend_setup.py:497-642)."""
        if self.movie_config.enabled:
            raise ValueError("movie-frame particle extraction is not supported by leopard_em_gb300")
        template = self.template_volume
        if template is None:
            template = self.template_volume = load_mrc_volume(self.template_volume_path)
        template = torch.as_tensor(template, dtype=torch.float32)
        ps = self.particle_stack
        h, w = ps.original_template_size
        box_h, box_w = ps.extracted_box_size
        crop = (box_h - h + 1, box_w - w + 1)
        # statistics maps of the search, cropped at every particle (backend_setup.py:318-370)
        avg, avg_idx = ps.load_images_grouped_by_column("correlation_average_path")
        corr_mean = ps.construct_image_stack(avg, avg_idx, crop, padding_value=0.0, padding_mode="constant")
        var, var_idx = ps.load_images_grouped_by_column("correlation_variance_path")
        corr_std = ps.construct_image_stack(var, var_idx, crop, padding_value=1e10, padding_mode="constant") ** 0.5
        # particle images and projective filters (backend_setup.py:373-490)
        mics, mic_idx = ps.load_images_grouped_by_column("micrograph_path")
        filt_shape = (template.shape[-2], template.shape[-1] // 2 + 1)
        pfilters = None
        if self.apply_global_filtering:
            img_h, img_w = mics.shape[-2:]
            mdft = torch.fft.rfftn(mics, dim=(-2, -1))
            mdft[..., 0, 0] = 0 + 0j
            pfilters = ps.construct_projective_filters(self.preprocessing_filters, filt_shape, mdft, mic_idx)
            mdft = self._apply_image_filtering(mdft, (img_h, img_w), (box_h + 1, box_w + 1))
            mics = torch.fft.irfftn(mdft, s=(img_h, img_w), dim=(-2, -1))
        parts = ps.construct_image_stack(mics, mic_idx, ps.extracted_box_size, padding_value=0.0,
                                         padding_mode="reflect")
        pdft = torch.fft.rfftn(parts, dim=(-2, -1))
        if not self.apply_global_filtering:
            pdft[..., 0, 0] = 0 + 0j
            pfilters = ps.construct_image_filters(self.preprocessing_filters, filt_shape, pdft)
            pdft = self._apply_image_filtering(pdft, (box_h, box_w), (box_h, box_w))
        defocus_u, defocus_v = ps.get_absolute_defocus()
        ctf_kwargs = ps.ctf_kwargs((template.shape[-2], template.shape[-1]))
        if ctf_kwargs["even_zernikes"] or ctf_kwargs["odd_zernikes"]:
            raise ValueError("Zernike aberration terms are not supported by leopard_em_gb300")
        return {
            "particle_stack_dft": pdft.to(torch.complex64),
            "template_dft": pp.volume_to_rfft_fourier_slice(template).to(torch.complex64),
            "euler_angles": ps.get_euler_angles(prefer_refined_angles).to(torch.float32),
            "euler_angle_offsets": self.orientation_refinement_config.euler_angles_offsets,
            "defocus_u": defocus_u.to(torch.float32),
            "defocus_v": defocus_v.to(torch.float32),
            "defocus_angle": torch.as_tensor(ps["astigmatism_angle"], dtype=torch.float32),
            "defocus_offsets": self.defocus_refinement_config.defocus_values,
            "pixel_size_offsets": self.pixel_size_refinement_config.pixel_size_values,
            "corr_mean": corr_mean.to(torch.float32),
            "corr_std": corr_std.to(torch.float32),
            "ctf_kwargs": ctf_kwargs,
            "projective_filters": pfilters.to(torch.float32),
            "device": self.computational_config.gpu_devices,
            "mag_matrix": ctf_kwargs["mag_matrix"],
        }

    def _apply_image_filtering(self, images_dft, full_image_shape, extracted_box_shape):
        """Per-image combined filter and unit-power normalisation
        (utils/image_processing.py:78-115)."""
        bp = self.preprocessing_filters.bandpass_filter.calculate_bandpass_filter(images_dft.shape[-2:],
                                                                                    device=images_dft.device)
        filters = self.particle_stack.construct_image_filters(self.preprocessing_filters,
                                                              tuple(images_dft.shape[-2:]), images_dft)
        return pp.preprocess_image(images_dft, filters, bp, full_image_shape, extracted_box_shape)

    def run_refine_template(self, orientation_batch_size: int = 64) -> dict:
        kw = self.make_backend_core_function_kwargs()
        return core_refine_template(**kw, batch_size=orientation_batch_size,
                                    num_cuda_streams=self.computational_config.num_cpus)

    def run_refine_template_learned(self, orientation_batch_size: int = 64, weights_path: Optional[str] = None,
                                    proposal: Literal["network", "gauss_newton"] = "network",
                                    small_offsets: Optional[torch.Tensor] = None,
                                    small_defocus: Optional[torch.Tensor] = None):
        """Refinement with learned proposals (no reference counterpart; see
        ``proposal.refine_with_proposals``): the proposal network (the shipped
        weights unless ``weights_path``) or the Gauss-Newton step proposes each
        particle's pose and defocus, a small plain grid around the proposal
        (default +-0.5 deg at 0.125 deg x +-100 A at 50 A) scores it, and every
        particle whose proposal does not beat its starting pose falls back to
        this manager's full plain grid.  Crops must be at least 128 x 128 (the
        network sees the 64 x 64 lowest-frequency band).

        Returns (result, info): ``result`` has the keys of
        ``run_refine_template``; ``info`` counts the fallbacks."""
        from . import proposal as pr
        from .backend.core_match_template import _single_cuda_device
        from .grids import local_euler_offsets

        box_h, box_w = self.particle_stack.extracted_box_size
        if box_h < 2 * pr.BAND or box_w < 2 * pr.BAND:
            raise ValueError(f"learned proposals need crops of at least {2 * pr.BAND} x {2 * pr.BAND}, "
                             f"got {box_h} x {box_w}; use run_refine_template")
        kw = self.make_backend_core_function_kwargs()
        dev = _single_cuda_device(kw.pop("device"))
        net = None
        if proposal == "network":
            path = weights_path or os.path.join(os.path.dirname(__file__), "weights", "proposal_refine288.npz")
            net = pr.load_net(path, dev)
        small = small_offsets if small_offsets is not None else local_euler_offsets(0.5, 0.125, 0.5, 0.125)
        small_df = small_defocus if small_defocus is not None else torch.arange(-100.0, 100.0 + 1e-6, 50.0)
        return pr.refine_with_proposals(net, kw, dev, small, small_df, batch_size=orientation_batch_size,
                                        proposal=proposal)

    def get_refine_result(self, backend_kwargs: dict, orientation_batch_size: int = 64) -> dict:
        """Refinement results as numpy arrays (refine_template_manager.py:314-353)."""
        res = core_refine_template(**backend_kwargs, batch_size=orientation_batch_size,
                                   num_cuda_streams=self.computational_config.num_cpus)
        return {k: (v.cpu().numpy() if isinstance(v, torch.Tensor) else v) for k, v in res.items()}

    def save_config(self, path: str, mode: Literal["yaml", "json"] = "yaml") -> None:
        if mode == "yaml":
            self.to_yaml(path)
        elif mode == "json":
            self.to_json(path)
        else:
            raise ValueError(f"Invalid serialization mode '{mode}'.")


__all__ = [
    "ArbitraryCurveFilterConfig", "BandpassFilterConfig", "ComputationalConfigMatch", "ComputationalConfigRefine",
    "DefocusSearchConfig", "MatchTemplateManager", "MatchTemplateResult", "MovieConfig",
    "MultipleOrientationConfig", "OpticsGroup", "OrientationSearchConfig", "ParticleStack",
    "PhaseRandomizationFilterConfig", "PixelSizeSearchConfig", "PreprocessingFilters", "RefineOrientationConfig",
    "RefineTemplateManager", "ValidationError", "WhiteningFilterConfig", "get_search_tensors",
]
