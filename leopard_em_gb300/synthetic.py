"""Seeded synthetic 2DTM workloads (stand-ins for the reference's benchmark data).

Every configuration is built from one integer seed:
  * template: a cubic volume that is a sum of isotropic Gaussian blobs
    (exp(-|r-c|^2 / 2 sigma^2)) with centres uniform in a ball;
  * micrograph: i.i.d. N(0,1) noise plus particles.  A particle is the exact
    line-integral projection of the blob volume at rotation R (blob centre c
    projects to (R^T c)_xy, the convention of the Fourier-slice search), CTF
    filtered, scaled so that its variance over the d x d box is ``snr`` times
    the noise variance, contrast inverted (the search flips the template
    contrast) and added with its box's top-left corner at a random position;
  * search inputs: preprocessed image spectrum, fftshifted template rfft, CTF
    stack, whitening filter, defocus and pixel-size offsets, Euler grid.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np
import torch

from . import preprocess as pp
from .grids import local_euler_offsets, uniform_euler_grid  # noqa: F401


def blob_volume(size: int, n_blobs: int, sigma: float, radius: float, seed: int, device="cpu"):
    """Sum of Gaussian blobs; returns (volume[z,y,x] float32, centres (n,3) xyz
    relative to voxel size//2)."""
    rng = np.random.default_rng(seed)
    # uniform in a ball
    v = rng.normal(size=(n_blobs, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    r = radius * rng.uniform(size=(n_blobs, 1)) ** (1.0 / 3.0)
    centres = v * r
    vol = torch.zeros((size, size, size), dtype=torch.float32, device=device)
    half = size // 2
    win = int(math.ceil(4 * sigma))
    offs = torch.arange(-win, win + 1, device=device, dtype=torch.float32)
    for cx, cy, cz in centres:
        ix, iy, iz = int(round(cx)) + half, int(round(cy)) + half, int(round(cz)) + half
        gx = torch.exp(-((offs + ix - half - cx) ** 2) / (2 * sigma**2))
        gy = torch.exp(-((offs + iy - half - cy) ** 2) / (2 * sigma**2))
        gz = torch.exp(-((offs + iz - half - cz) ** 2) / (2 * sigma**2))
        blk = gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
        z0, y0, x0 = iz - win, iy - win, ix - win
        zs, ys, xs = max(z0, 0), max(y0, 0), max(x0, 0)
        ze, ye, xe = min(z0 + 2 * win + 1, size), min(y0 + 2 * win + 1, size), min(x0 + 2 * win + 1, size)
        if ze <= zs or ye <= ys or xe <= xs:
            continue
        vol[zs:ze, ys:ye, xs:xe] += blk[zs - z0 : ze - z0, ys - y0 : ye - y0, xs - x0 : xe - x0]
    return vol, centres


def euler_zyz_from_rotmat(R: np.ndarray) -> np.ndarray:
    """(phi, theta, psi) in degrees with R = Rz(phi) Ry(theta) Rz(psi)."""
    theta = math.degrees(math.acos(max(-1.0, min(1.0, R[2, 2]))))
    if abs(R[2, 2]) < 1 - 1e-9:
        phi = math.degrees(math.atan2(R[1, 2], R[0, 2]))
        psi = math.degrees(math.atan2(R[2, 1], -R[2, 0]))
    else:
        phi = math.degrees(math.atan2(R[1, 0], R[0, 0]))
        psi = 0.0
    return np.array([phi % 360.0, theta, psi % 360.0])


def random_euler_angles(n: int, seed: int = 0) -> torch.Tensor:
    """(n, 3) float32 ZYZ Euler angles (degrees) of rotations drawn uniformly
    from SO(3) (normalised Gaussian quaternions), seeded."""
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)
    return torch.tensor(np.stack([euler_zyz_from_rotmat(r) for r in R]), dtype=torch.float32)


def rotmat_zyz(euler_deg) -> np.ndarray:
    phi, theta, psi = (math.radians(a) for a in euler_deg)

    def rz(a):
        return np.array([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1]])

    def ry(a):
        return np.array([[math.cos(a), 0, math.sin(a)], [0, 1, 0], [-math.sin(a), 0, math.cos(a)]])

    return rz(phi) @ ry(theta) @ rz(psi)


def project_blobs(centres: np.ndarray, sigma: float, rot: np.ndarray, size: int, device="cpu") -> torch.Tensor:
    """Exact line-integral projection (size x size, [y, x]) of the blob volume at rot."""
    p = torch.tensor(centres @ rot, dtype=torch.float64, device=device)  # rows = (R^T c)^T
    g = torch.arange(size, dtype=torch.float64, device=device) - size // 2
    gx = torch.exp(-((g[None, :] - p[:, 0:1]) ** 2) / (2 * sigma**2))
    gy = torch.exp(-((g[None, :] - p[:, 1:2]) ** 2) / (2 * sigma**2))
    return (math.sqrt(2 * math.pi) * sigma * (gy.T @ gx)).to(torch.float32)


@dataclass
class MatchConfig:
    image_shape: tuple[int, int] = (512, 512)
    template_size: int = 64
    n_blobs: int = 200
    blob_sigma: float = 1.5
    blob_radius: float = 24.0
    pixel_size: float = 1.0
    n_particles: int = 20
    snr: float = 0.3
    voltage: float = 300.0
    spherical_aberration: float = 2.7
    amplitude_contrast: float = 0.07
    defocus: float = 12000.0
    defocus_offsets: tuple[float, ...] = (0.0,)
    pixel_size_offsets: tuple[float, ...] = (0.0,)
    out_of_plane_step: float = 20.0
    in_plane_step: float = 20.0
    orientation_batch: int = 8
    plant_from_grid: bool = True
    seed: int = 0
    name: str = "custom"


# The two single-micrograph configurations of the plain method.
CONFIG_SMALL = MatchConfig(name="2dtm-512sq-64cube-20deg")
CONFIG_PRODUCTION = MatchConfig(
    image_shape=(4096, 4096),
    template_size=384,
    n_blobs=4000,
    blob_sigma=1.2,
    blob_radius=150.0,
    pixel_size=1.06,
    n_particles=300,
    snr=0.1,
    defocus=10000.0,
    defocus_offsets=(-200.0, 0.0, 200.0),
    out_of_plane_step=2.5,
    in_plane_step=1.5,
    orientation_batch=8,
    plant_from_grid=False,
    name="2dtm-4096sq-384cube-2.5deg-1.5deg-3df",
)


# The shape of the reference's published benchmark (4096^2 micrograph, 512^3
# template, 11 defocus planes), for a like-for-like correlograms/s figure.
CONFIG_REFBENCH = MatchConfig(
    image_shape=(4096, 4096),
    template_size=512,
    n_blobs=6000,
    blob_sigma=1.2,
    blob_radius=200.0,
    pixel_size=1.06,
    n_particles=100,
    snr=0.1,
    defocus=10000.0,
    defocus_offsets=tuple(float(x) for x in range(-500, 501, 100)),
    out_of_plane_step=2.5,
    in_plane_step=1.5,
    orientation_batch=8,
    plant_from_grid=False,
    name="2dtm-4096sq-512cube-2.5deg-1.5deg-11df",
)


@dataclass
class MatchWorkload:
    config: MatchConfig
    kwargs: dict
    planted: list = field(default_factory=list)  # (y0, x0, orientation index or -1, euler)
    image: torch.Tensor | None = None


def make_template(cfg: MatchConfig, device="cpu"):
    """(template_dft on the CPU, blob centres) of ``cfg``'s Gaussian-blob volume."""
    vol, centres = blob_volume(cfg.template_size, cfg.n_blobs, cfg.blob_sigma, cfg.blob_radius, cfg.seed,
                               device=device)
    template_dft = pp.volume_to_rfft_fourier_slice(vol).cpu()
    return template_dft, centres


def make_match_workload(cfg: MatchConfig, device="cpu", keep_image: bool = False,
                        euler_angles: torch.Tensor | None = None, template=None) -> MatchWorkload:
    """Build the ``core_match_template`` keyword arguments for ``cfg`` (CPU tensors).

    ``template`` = (template_dft, centres) from ``make_template`` reuses one
    volume across micrographs (its blob parameters must be ``cfg``'s)."""
    H, W = cfg.image_shape
    d = cfg.template_size
    rng = np.random.default_rng(cfg.seed + 1)
    template_dft, centres = make_template(cfg, device) if template is None else template
    if euler_angles is None:
        euler_angles = uniform_euler_grid(cfg.out_of_plane_step, cfg.in_plane_step)
    gen = torch.Generator(device="cpu").manual_seed(cfg.seed + 2)
    image = torch.randn((H, W), generator=gen, dtype=torch.float32).to(device)
    box_ctf = pp.ctf_2d((d, d), cfg.defocus, 0.0, 0.0, cfg.voltage, cfg.spherical_aberration,
                        cfg.amplitude_contrast, 0.0, cfg.pixel_size).to(device)
    planted = []
    for _ in range(cfg.n_particles):
        if cfg.plant_from_grid:
            oi = int(rng.integers(euler_angles.shape[0]))
            eul = euler_angles[oi].double().numpy()
        else:
            oi = -1
            q = rng.normal(size=4)
            q /= np.linalg.norm(q)
            w, x, y, z = q
            Rq = np.array([
                [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
            ])
            eul = euler_zyz_from_rotmat(Rq)
        proj = project_blobs(centres, cfg.blob_sigma, rotmat_zyz(eul), d, device=device)
        proj = torch.fft.irfft2(torch.fft.rfft2(proj) * box_ctf, s=(d, d))
        proj = proj - proj.mean()
        proj = proj * (math.sqrt(cfg.snr) / proj.std().clamp_min(1e-12))
        y0 = int(rng.integers(0, H - d + 1))
        x0 = int(rng.integers(0, W - d + 1))
        image[y0 : y0 + d, x0 : x0 + d] -= proj
        planted.append((y0, x0, oi, tuple(float(a) for a in eul)))
    image_dft = torch.fft.rfftn(image)
    image_dft[0, 0] = 0 + 0j
    wf_img = pp.whitening_filter(image_dft.cpu(), (H, W)).to(device)
    wf_tmp = pp.whitening_filter(image_dft.cpu(), (d, d))
    bandpass = torch.ones_like(wf_img)
    image_dft = pp.preprocess_image(image_dft, wf_img, bandpass, (H, W), (H, W)).cpu()
    defocus_offsets = torch.tensor(cfg.defocus_offsets, dtype=torch.float32)
    pixel_offsets = torch.tensor(cfg.pixel_size_offsets, dtype=torch.float32)
    ctf = pp.ctf_filter_stack(d, cfg.defocus, cfg.defocus, defocus_offsets, pixel_offsets,
                              voltage=cfg.voltage, spherical_aberration=cfg.spherical_aberration,
                              amplitude_contrast=cfg.amplitude_contrast, pixel_size=cfg.pixel_size)
    kwargs = dict(
        image_dft=image_dft.to(torch.complex64),
        template_dft=template_dft.to(torch.complex64),
        ctf_filters=ctf,
        whitening_filter_template=wf_tmp,
        defocus_values=defocus_offsets,
        pixel_values=pixel_offsets,
        euler_angles=euler_angles,
    )
    return MatchWorkload(cfg, kwargs, planted, image.cpu() if keep_image else None)


# Batched form: micrographs of uneven sizes, one 256^3 template, 7 defocus
# planes x 3 pixel sizes, grid 3.0 / 2.0 degrees (825,480 orientations).
BATCHED_SIZES = ((2048, 2048), (3072, 2880), (3838, 3710), (4096, 4096), (5760, 4092))
CONFIG_BATCHED = MatchConfig(
    image_shape=(4096, 4096),
    template_size=256,
    n_blobs=2000,
    blob_sigma=1.2,
    blob_radius=100.0,
    pixel_size=1.0,
    n_particles=150,
    snr=0.1,
    defocus=10000.0,
    defocus_offsets=(-600.0, -400.0, -200.0, 0.0, 200.0, 400.0, 600.0),
    pixel_size_offsets=(-0.02, 0.0, 0.02),
    out_of_plane_step=3.0,
    in_plane_step=2.0,
    orientation_batch=8,
    plant_from_grid=False,
    name="2dtm-batched-12-micrographs-256cube-3deg-2deg-7df-3px",
)


def batched_micrograph_configs(n_micrographs: int = 12, base: MatchConfig = CONFIG_BATCHED, seed: int = 0):
    """Per-micrograph configurations of the batched form: sizes cycle through
    ``BATCHED_SIZES``; 50-300 particles and SNR 0.05-0.2 drawn from the seed."""
    rng = np.random.default_rng(seed + 17)
    out = []
    for i in range(n_micrographs):
        out.append(replace(base, image_shape=BATCHED_SIZES[i % len(BATCHED_SIZES)],
                           n_particles=int(rng.integers(50, 301)), snr=float(rng.uniform(0.05, 0.2)),
                           seed=base.seed + 1000 * (i + 1), name=f"{base.name}/{i}"))
    return out


def make_batched_workload(n_micrographs: int = 12, device="cpu", base: MatchConfig = CONFIG_BATCHED,
                          euler_angles: torch.Tensor | None = None):
    """(template_dft, euler_angles, [per-micrograph kwargs], configs) of the batched form."""
    template = make_template(base, device)
    if euler_angles is None:
        euler_angles = uniform_euler_grid(base.out_of_plane_step, base.in_plane_step)
    mics, cfgs = [], batched_micrograph_configs(n_micrographs, base)
    for cfg in cfgs:
        wl = make_match_workload(cfg, device=device, euler_angles=euler_angles, template=template)
        kw = wl.kwargs
        mics.append({k: kw[k] for k in ("image_dft", "ctf_filters", "whitening_filter_template", "defocus_values",
                                         "pixel_values")})
    return template[0], euler_angles, mics, cfgs


@dataclass
class RefineConfig:
    crop: int = 288
    template_size: int = 256
    n_blobs: int = 4000
    blob_sigma: float = 1.2
    blob_radius: float = 100.0
    pixel_size: float = 1.06
    snr_range: tuple[float, float] = (0.05, 0.2)
    shift_px: float = 3.0
    defocus: float = 10000.0
    defocus_jitter: float = 400.0
    pose_perturbation_deg: float = 3.0
    grid_angle_range: float = 3.0
    grid_angle_step: float = 0.25
    grid_defocus_range: float = 400.0
    grid_defocus_step: float = 50.0
    batch: int = 32
    seed: int = 0
    name: str = "refine-288sq-256cube-3deg@0.25-400A@50"


CONFIG_REFINE = RefineConfig()


def random_rotations(n: int, gen: torch.Generator) -> torch.Tensor:
    """(n, 3, 3) float64 rotations, uniform on SO(3) (unit quaternions)."""
    q = torch.randn(n, 4, generator=gen, dtype=torch.float64)
    q = q / q.norm(dim=1, keepdim=True)
    w, x, y, z = q.unbind(1)
    return torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w),
        2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w),
        2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y),
    ], dim=1).reshape(n, 3, 3)


def axis_angle_rotations(axes: torch.Tensor, angles_rad: torch.Tensor) -> torch.Tensor:
    a = axes / axes.norm(dim=1, keepdim=True)
    K = torch.zeros(a.shape[0], 3, 3, dtype=a.dtype)
    K[:, 0, 1], K[:, 0, 2], K[:, 1, 0] = -a[:, 2], a[:, 1], a[:, 2]
    K[:, 1, 2], K[:, 2, 0], K[:, 2, 1] = -a[:, 0], -a[:, 1], a[:, 0]
    s, c = angles_rad.sin()[:, None, None], angles_rad.cos()[:, None, None]
    return torch.eye(3, dtype=a.dtype) + s * K + (1 - c) * (K @ K)


def simulate_particles(cfg: "RefineConfig", centres: np.ndarray, n: int, seed: int, device="cpu", chunk: int = 32):
    """Particles the method simulates: exact blob-volume projection at a random
    pose R_true, sub-pixel shift, defocus offset ddf, CTF, additive N(0,1)
    noise at a random SNR (signal variance / noise variance over the d x d box),
    contrast inverted, preprocessed like the search input.  Starting poses
    R_start = D^T R_true with D a rotation by U(0, max) degrees about a random
    axis.  Returns a dict of tensors (particle_dft on `device`, the rest CPU)."""
    gen = torch.Generator().manual_seed(seed)
    d, H = cfg.template_size, cfg.crop
    o = (H - d) // 2
    r_true = random_rotations(n, gen)
    axes = torch.randn(n, 3, generator=gen, dtype=torch.float64)
    ang = torch.rand(n, generator=gen, dtype=torch.float64) * math.radians(cfg.pose_perturbation_deg)
    dmat = axis_angle_rotations(axes, ang)
    r_start = dmat.transpose(1, 2) @ r_true
    ddf = (torch.rand(n, generator=gen, dtype=torch.float64) * 2 - 1) * cfg.defocus_jitter
    shift = (torch.rand(n, 2, generator=gen, dtype=torch.float64) * 2 - 1) * cfg.shift_px
    lo, hi = cfg.snr_range
    snr = lo + (hi - lo) * torch.rand(n, generator=gen, dtype=torch.float64)
    noise_seeds = torch.randint(0, 1 << 30, (n,), generator=gen)
    dev = torch.device(device)
    cen = torch.tensor(centres, dtype=torch.float32, device=dev)
    g1 = torch.arange(d, dtype=torch.float32, device=dev) - d // 2
    ky = (torch.fft.fftfreq(H, dtype=torch.float64, device=dev)[:, None] / cfg.pixel_size)
    kx = (torch.fft.rfftfreq(H, dtype=torch.float64, device=dev)[None, :] / cfg.pixel_size)
    k2 = kx**2 + ky**2
    lam = pp.electron_wavelength(300.0)
    k5 = math.atan(0.07 / math.sqrt(1 - 0.07**2))
    chi_static = 0.5 * math.pi * 2.7e7 * lam**3 * k2**2 - k5
    amp = math.sqrt(2 * math.pi) * cfg.blob_sigma
    out = torch.empty((n, H, H // 2 + 1), dtype=torch.complex64, device=dev)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        R = r_true[a:b].to(dev, torch.float32)
        pxy = cen[None] @ R                       # (m, nb, 3): rows (R^T c)^T
        gx = torch.exp(-((g1[None, None, :] - pxy[:, :, 0:1]) ** 2) / (2 * cfg.blob_sigma**2))
        gy = torch.exp(-((g1[None, None, :] - pxy[:, :, 1:2]) ** 2) / (2 * cfg.blob_sigma**2))
        proj = amp * (gy.transpose(1, 2) @ gx)    # (m, d, d)
        box = torch.zeros((b - a, H, H), dtype=torch.float32, device=dev)
        box[:, o : o + d, o : o + d] = proj
        f = torch.fft.rfft2(box.double())
        sh = shift[a:b].to(dev)
        f = f * torch.exp(-2j * math.pi * (ky[None] * sh[:, 0, None, None] + kx[None] * sh[:, 1, None, None]))
        df = (cfg.defocus + ddf[a:b]).to(dev)
        chi = -math.pi * lam * k2[None] * df[:, None, None] + chi_static[None]
        f = f * (-torch.sin(chi))
        sig = torch.fft.irfft2(f, s=(H, H))
        sig = sig - sig.mean(dim=(1, 2), keepdim=True)
        sd = sig[:, o : o + d, o : o + d].std(dim=(1, 2), keepdim=True).clamp_min(1e-12)
        sig = sig * (snr[a:b].to(dev).sqrt()[:, None, None] / sd)
        ngen = torch.Generator(device=dev).manual_seed(int(noise_seeds[a]))
        noise = torch.randn((b - a, H, H), generator=ngen, dtype=torch.float64, device=dev)
        img = (noise - sig).to(torch.float32)
        fi = torch.fft.rfftn(img, dim=(1, 2))
        fi[:, 0, 0] = 0
        sq = fi.abs() ** 2
        ssum = sq.sum(dim=(1, 2), keepdim=True) + sq[:, :, 1:-1].sum(dim=(1, 2), keepdim=True)
        dim_ = H * (H // 2 + 1) + H * (H // 2 - 1)  # all-ones bandpass dimensionality
        out[a:b] = (fi / torch.sqrt(ssum) * math.sqrt(dim_)).to(torch.complex64)
    return {"particle_dft": out, "r_true": r_true, "r_start": r_start, "ddf": ddf, "shift": shift, "snr": snr}


def make_refine_workload(cfg: "RefineConfig", n_particles: int, device="cpu", grid: torch.Tensor | None = None,
                         seed_offset: int = 0):
    """``core_refine_template`` keyword arguments for n simulated particles
    (starting poses perturbed, defocus at the nominal value), plus the truth."""
    from .rotations import rotmat_to_euler_zyz

    d, H = cfg.template_size, cfg.crop
    vol, centres = blob_volume(d, cfg.n_blobs, cfg.blob_sigma, cfg.blob_radius, cfg.seed, device=device)
    template_dft = pp.volume_to_rfft_fourier_slice(vol).cpu().to(torch.complex64)
    del vol
    sim = simulate_particles(cfg, centres, n_particles, cfg.seed + 11 + seed_offset, device=device)
    crop = H - d + 1
    if grid is None:
        grid = local_euler_offsets(cfg.grid_angle_range, cfg.grid_angle_step, cfg.grid_angle_range,
                                   cfg.grid_angle_step)
    dfs = torch.arange(-cfg.grid_defocus_range, cfg.grid_defocus_range + 1e-6, cfg.grid_defocus_step,
                       dtype=torch.float32)
    kwargs = dict(
        particle_stack_dft=sim["particle_dft"].cpu(),
        template_dft=template_dft,
        euler_angles=rotmat_to_euler_zyz(sim["r_start"]).to(torch.float32),
        euler_angle_offsets=grid,
        defocus_offsets=dfs,
        defocus_u=torch.full((n_particles,), cfg.defocus),
        defocus_v=torch.full((n_particles,), cfg.defocus),
        defocus_angle=torch.zeros(n_particles),
        pixel_size_offsets=torch.zeros(1),
        corr_mean=torch.zeros(n_particles, crop, crop),
        corr_std=torch.ones(n_particles, crop, crop),
        ctf_kwargs=dict(voltage=300.0, spherical_aberration=2.7, amplitude_contrast_ratio=0.07, ctf_B_factor=0.0,
                        phase_shift=0.0, pixel_size=cfg.pixel_size, template_shape=(d, d), even_zernikes=None,
                        odd_zernikes=None, mag_matrix=None),
        projective_filters=torch.ones(n_particles, d, d // 2 + 1),
    )
    truth = {k: v for k, v in sim.items() if k != "particle_dft"}
    truth["centres"] = centres
    return kwargs, truth
