"""Particle table + image extraction for the refinement manager.

Mirrors Leopard-EM's ``ParticleStack`` (pydantic_models/data_structures/
particle_stack.py:292-880): a CSV table of particles found by the search (one
row per particle, the columns of ``MATCH_TEMPLATE_DF_COLUMN_ORDER``,
pydantic_models/formats.py:3-43) plus the box sizes used to cut particle
images, correlation-statistics crops and per-micrograph filters out of the
referenced MRC files.  The table is held as named columns (numpy arrays for
numbers, lists for text) instead of a pandas DataFrame; the methods keep the
reference's names, arguments and fallbacks (refined columns first, unrefined
ones with a warning).
"""

from __future__ import annotations

import csv
import json
import math
import warnings
from typing import Any, Literal

import numpy as np
import torch
import torch.nn.functional as F

from .config_models import ConfigModel, Field

# The columns a search writes per particle (a file format: same names and order
# as the reference's MATCH_TEMPLATE_DF_COLUMN_ORDER).
MATCH_TEMPLATE_DF_COLUMN_ORDER = [
    "particle_index", "mip", "scaled_mip", "correlation_mean", "correlation_variance", "total_correlations",
    "pos_x", "pos_y", "pos_x_img", "pos_y_img", "pos_x_img_angstrom", "pos_y_img_angstrom", "phi", "theta", "psi",
    "relative_defocus", "defocus_u", "defocus_v", "astigmatism_angle", "pixel_size", "refined_pixel_size",
    "voltage", "spherical_aberration", "amplitude_contrast_ratio", "phase_shift", "ctf_B_factor", "even_zernikes",
    "odd_zernikes", "mag_matrix", "micrograph_path", "template_path", "mip_path", "scaled_mip_path", "psi_path",
    "theta_path", "phi_path", "defocus_path", "correlation_average_path", "correlation_variance_path",
]


def _parse(v: str):
    if v is None or v == "" or v.lower() in ("nan", "none", "null"):
        return float("nan")
    try:
        return float(v)
    except ValueError:
        return v


def read_particle_table(path) -> dict:
    """CSV -> {column: numpy float array | list of str}."""
    with open(path, newline="", encoding="utf-8") as f:
        rows = list(csv.DictReader(f))
    if not rows:
        raise ValueError(f"particle table '{path}' has no rows")
    cols = {}
    for name in rows[0].keys():
        vals = [_parse(r[name]) for r in rows]
        if all(isinstance(v, float) for v in vals):
            cols[name] = np.asarray(vals, dtype=np.float64)
        else:
            cols[name] = [None if isinstance(v, float) and math.isnan(v) else (v if isinstance(v, str) else repr(v))
                          for v in vals]
    return cols


def write_particle_table(path, columns: dict) -> None:
    """{column: sequence} -> CSV (the inverse of ``read_particle_table``)."""
    names = list(columns)
    n = len(next(iter(columns.values())))
    with open(path, "w", newline="", encoding="utf-8") as f:
        w = csv.writer(f)
        w.writerow(names)
        for i in range(n):
            row = []
            for k in names:
                v = columns[k][i]
                if isinstance(v, (list, dict)):
                    v = json.dumps(v)
                row.append("" if v is None else v)
            w.writerow(row)


def _nan_or_inf(a) -> bool:
    return not isinstance(a, np.ndarray) or bool(np.any(~np.isfinite(a)))


def get_cropped_image_regions(image: torch.Tensor, pos_y, pos_x, box_size, handle_bounds: str = "pad",
                              padding_mode: str = "constant", padding_value: float = 0.0) -> torch.Tensor:
    """(N, box_h, box_w) boxes whose top-left corners are (pos_y, pos_x); boxes
    reaching outside the image are padded (constant / reflect / replicate) or
    rejected (particle_stack.py:52-289)."""
    box_h, box_w = box_size
    H, W = image.shape[-2:]
    py = np.asarray(pos_y, dtype=np.int64).reshape(-1)
    px = np.asarray(pos_x, dtype=np.int64).reshape(-1)
    if py.size == 0:
        return image.new_zeros((0, box_h, box_w))
    top = int(max(0, -py.min()))
    bottom = int(max(0, py.max() + box_h - H))
    left = int(max(0, -px.min()))
    right = int(max(0, px.max() + box_w - W))
    if handle_bounds == "error" and (top or bottom or left or right):
        raise ValueError("particle boxes extend beyond the image bounds")
    if handle_bounds not in ("pad", "error"):
        raise ValueError(f"handle_bounds must be 'pad' or 'error', got {handle_bounds!r}")
    img = image
    if top or bottom or left or right:
        if padding_mode == "constant":
            img = F.pad(image[None, None], (left, right, top, bottom), mode="constant", value=padding_value)[0, 0]
        elif padding_mode in ("reflect", "replicate"):
            img = F.pad(image[None, None], (left, right, top, bottom), mode=padding_mode)[0, 0]
        else:
            raise ValueError(f"padding_mode must be constant, reflect or replicate, got {padding_mode!r}")
    out = torch.empty((py.size, box_h, box_w), dtype=image.dtype, device=image.device)
    for i, (y, x) in enumerate(zip(py.tolist(), px.tolist())):
        out[i] = img[y + top:y + top + box_h, x + left:x + left + box_w]
    return out


class ParticleStack(ConfigModel):
    df_path: str
    extracted_box_size: tuple[int, int]
    original_template_size: tuple[int, int]
    image_stack: Any = Field(None, exclude=True)

    def __init__(self, skip_df_load: bool = False, **data: Any):
        super().__init__(**data)
        object.__setattr__(self, "_df", {})
        if not skip_df_load:
            self.load_df()

    def validate(self) -> None:
        if self.extracted_box_size[0] <= self.original_template_size[0] or \
                self.extracted_box_size[1] <= self.original_template_size[1]:
            raise ValueError("extracted_box_size must be larger than original_template_size "
                             f"({self.extracted_box_size} vs {self.original_template_size})")

    # -- table -------------------------------------------------------------
    def load_df(self) -> None:
        cols = read_particle_table(self.df_path)
        missing = [c for c in MATCH_TEMPLATE_DF_COLUMN_ORDER if c not in cols]
        if missing:
            raise ValueError(f"Missing the following columns in DataFrame: {missing}")
        object.__setattr__(self, "_df", cols)

    @property
    def df_columns(self) -> list[str]:
        return list(self._df)

    @property
    def num_particles(self) -> int:
        return len(next(iter(self._df.values()))) if self._df else 0

    def __getitem__(self, key: str):
        if key not in self._df:
            raise KeyError(f"Column '{key}' not found in the particle table.")
        return self._df[key]

    def set_column(self, column_name: str, value: Any) -> None:
        if isinstance(value, torch.Tensor):
            value = value.detach().cpu().numpy()
        if np.isscalar(value):
            value = np.full(self.num_particles, value, dtype=np.float64)
        arr = np.asarray(value) if not isinstance(value, list) else value
        if len(arr) != self.num_particles:
            raise ValueError(f"column '{column_name}' needs {self.num_particles} values, got {len(arr)}")
        self._df[column_name] = arr

    def get_dataframe_copy(self) -> dict:
        return {k: (v.copy() if isinstance(v, np.ndarray) else list(v)) for k, v in self._df.items()}

    def _numeric(self, col: str) -> np.ndarray:
        v = self._df[col]
        if not isinstance(v, np.ndarray):
            raise ValueError(f"column '{col}' is not numeric")
        return v

    def _get_position_reference_columns(self) -> tuple[str, str]:
        y = "refined_pos_y" if "refined_pos_y" in self._df else "pos_y"
        x = "refined_pos_x" if "refined_pos_x" in self._df else "pos_x"
        return y, x

    # -- images ------------------------------------------------------------
    def load_images_grouped_by_column(self, column_name: str):
        """Unique images of ``column_name`` (sorted by path, as a group-by) and,
        per image, the row indices of its particles."""
        from .managers import load_mrc_image

        if column_name not in self._df:
            raise ValueError(f"Column '{column_name}' not found in the DataFrame.")
        paths = self._df[column_name]
        groups: dict[str, list[int]] = {}
        for i, p in enumerate(paths):
            groups.setdefault(str(p), []).append(i)
        images, indices = [], []
        for p in sorted(groups):
            images.append(load_mrc_image(p))
            indices.append(np.asarray(groups[p], dtype=np.int64))
        return torch.stack(images, dim=0), indices

    def construct_image_stack(self, images: torch.Tensor, indices, extraction_size,
                              pos_reference: Literal["center", "top-left"] = "top-left",
                              handle_bounds: Literal["pad", "error"] = "pad",
                              padding_mode: Literal["constant", "reflect", "replicate"] = "constant",
                              padding_value: float = 0.0) -> torch.Tensor:
        """Boxes of ``extraction_size`` around every particle
        (particle_stack.py:440-590): the box's top-left corner is the
        particle's position (the template corner) moved up-left by half the
        margin (box - template) // 2."""
        y_col, x_col = self._get_position_reference_columns()
        h, w = self.original_template_size
        box_h, box_w = self.extracted_box_size
        if images.shape[0] != len(indices):
            raise ValueError(f"Number of images ({images.shape[0]}) does not match the number of indices "
                             f"({len(indices)}).")
        stack = torch.zeros((self.num_particles, *extraction_size), device=images.device, dtype=images.dtype)
        for i, idx in enumerate(indices):
            py = self._numeric(y_col)[idx].astype(np.int64)
            px = self._numeric(x_col)[idx].astype(np.int64)
            if pos_reference == "center":
                py, px = py - h // 2, px - w // 2
            py = py - (box_h - h) // 2
            px = px - (box_w - w) // 2
            stack[torch.as_tensor(idx, device=images.device)] = get_cropped_image_regions(
                images[i], py, px, extraction_size, handle_bounds, padding_mode, padding_value)
        self.image_stack = stack
        return stack

    def construct_image_filters(self, preprocess_filters, output_shape, images_dft: torch.Tensor) -> torch.Tensor:
        out = torch.zeros((images_dft.shape[0], *output_shape), device=images_dft.device)
        for i in range(images_dft.shape[0]):
            out[i] = preprocess_filters.get_combined_filter(images_dft[i], tuple(output_shape))
        return out

    def construct_projective_filters(self, preprocess_filters, output_shape, images_dft: torch.Tensor,
                                     indices) -> torch.Tensor:
        if images_dft.shape[0] != len(indices):
            raise ValueError(f"Number of images ({images_dft.shape[0]}) does not match the number of indices "
                             f"({len(indices)}).")
        out = torch.zeros((self.num_particles, *output_shape), device=images_dft.device)
        for i, idx in enumerate(indices):
            out[torch.as_tensor(idx, device=images_dft.device)] = preprocess_filters.get_combined_filter(
                images_dft[i], tuple(output_shape))
        return out

    # -- per-particle parameters ---------------------------------------------
    def _prefer(self, refined: str, plain: str, prefer: bool, what: str) -> str:
        if not prefer:
            return plain
        if refined not in self._df:
            warnings.warn(f"Refined {what} not found in DataFrame, using original {what}...", stacklevel=3)
            return plain
        if _nan_or_inf(self._df[refined]):
            warnings.warn(f"Refined {what} contain NaN or inf values, using original {what}...", stacklevel=3)
            return plain
        return refined

    def get_relative_defocus(self, prefer_refined_defocus: bool = True) -> torch.Tensor:
        col = self._prefer("refined_relative_defocus", "relative_defocus", prefer_refined_defocus, "defocus values")
        return torch.tensor(self._numeric(col).copy())

    def get_absolute_defocus(self, prefer_refined_defocus: bool = True):
        rel = self.get_relative_defocus(prefer_refined_defocus)
        return (torch.tensor(self._numeric("defocus_u").copy()) + rel,
                torch.tensor(self._numeric("defocus_v").copy()) + rel)

    def get_pixel_size(self, prefer_refined_pixel_size: bool = True) -> torch.Tensor:
        col = self._prefer("refined_pixel_size", "pixel_size", prefer_refined_pixel_size, "pixel size")
        return torch.tensor(self._numeric(col).copy())

    def get_euler_angles(self, prefer_refined_angles: bool = True) -> torch.Tensor:
        cols = ("phi", "theta", "psi")
        if prefer_refined_angles:
            if all(f"refined_{c}" in self._df for c in cols):
                cols = tuple(f"refined_{c}" for c in cols)
            else:
                warnings.warn("Refined angles not found in DataFrame, using original angles...", stacklevel=2)
        return torch.stack([torch.tensor(self._numeric(c).copy()) for c in cols], dim=-1)

    def ctf_kwargs(self, template_shape) -> dict:
        """CTF parameters shared by every particle (utils/ctf_utils.py:202-262):
        one value per column across the stack, pixel size = mean refined pixel
        size, optional mag_matrix / Zernike terms parsed from their text."""
        for col in ("voltage", "spherical_aberration", "amplitude_contrast_ratio", "phase_shift", "ctf_B_factor"):
            if np.unique(self._numeric(col)).size != 1:
                raise ValueError(f"'{col}' must be the same for every particle")

        def first_text(col):
            vals = self._df[col]
            if isinstance(vals, np.ndarray):
                return None if np.all(np.isnan(vals)) else vals[0]
            uniq = {v for v in vals}
            if len(uniq) > 1:
                raise ValueError(f"'{col}' must be the same for every particle")
            return vals[0]

        mag = first_text("mag_matrix")
        mag_t = None
        if mag is not None:
            m = [float(x) for x in str(mag).strip("[]").split(",")] if isinstance(mag, str) else list(mag)
            if len(m) != 4:
                raise ValueError("mag_matrix must have 4 values")
            mag_t = torch.tensor([[m[0], m[1]], [m[2], m[3]]], dtype=torch.float32)

        def zern(col):
            v = first_text(col)
            if v is None:
                return None
            d = json.loads(v) if isinstance(v, str) else v
            return {k: torch.tensor(x, dtype=torch.float32) for k, x in d.items()} if d else None

        return {"voltage": float(self._numeric("voltage")[0]),
                "spherical_aberration": float(self._numeric("spherical_aberration")[0]),
                "amplitude_contrast_ratio": float(self._numeric("amplitude_contrast_ratio")[0]),
                "ctf_B_factor": float(self._numeric("ctf_B_factor")[0]),
                "phase_shift": float(self._numeric("phase_shift")[0]),
                "pixel_size": float(np.mean(self._numeric("refined_pixel_size"))),
                "template_shape": tuple(template_shape),
                "even_zernikes": zern("even_zernikes"), "odd_zernikes": zern("odd_zernikes"), "mag_matrix": mag_t}
