#!/usr/bin/env python
"""Throughput of the plain FP32 2DTM whole-orientation search on one GB300.

Workload (production configuration): 4096 x 4096 micrograph (N(0,1) noise +
300 planted projections at SNR 0.1), 384^3 Gaussian-blob template at
1.06 A/px, 3 defocus planes (-200/0/+200 A around 10000 A), orientation grid
2.5 deg out-of-plane / 1.5 deg in-plane (~1.58 M orientations), orientation
batch 64 (the autotuner's choice for a 4096^2 grid, and the fastest measured:
4,543 against 4,525 at 48, 4,482 at 32 and 4,351 at 16 orientations/s).  All
inputs are synthetic and seeded.

One "step" = one chunk of ``--orient-per-step`` consecutive orientations of
the grid (default 192 = 3 batches of 64 = 576 cross-correlograms), folded into
the running statistics maps, exactly as one slice of a full search.
``value``      orientations/s with inputs resident in HBM (device-timed, CUDA
               events on the launching stream); every batch streams a 12.9 GB
               correlogram intermediate, far larger than the 129 MB L2.
``e2e``        the same metric through the public drop-in
               ``core_match_template`` called with pinned host tensors: every
               call uploads its inputs, searches a slice of ``--e2e-orient``
               orientations (default 1536), finalises and copies the result
               maps back to the host.
``roofline``   the dominant kernel's algorithmic HBM bytes per launch over its
               mean event-timed duration, against the measured copy bandwidth.
``cpu_baseline`` the CPU oracle (a restatement of the reference's CPU path,
               torch.fft/pocketfft) on the host cores, on a bounded sample.
``--impl reference`` times that CPU implementation as the reference arm.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "orientations/s on 4096² image vs plain FP32 kernels; refined particles/s at equal SNR"
UNIT = "orientations/s"


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--orient-per-step", type=int, default=192)
    ap.add_argument("--e2e-steps", type=int, default=6)
    ap.add_argument("--e2e-orient", type=int, default=1536,
                    help="orientations per end-to-end call (a slice of the grid, as a caller splitting the search)")
    ap.add_argument("--cpu-sample-orient", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--config", choices=["production", "small", "refbench"], default="production",
                    help="refbench: the reference's published benchmark shape (4096^2, 512^3, 11 defocus)")
    ap.add_argument("--batch", type=int, default=-1,
                    help="orientation batch (0: the configuration's; -1: 64 for the production and reference-"
                         "benchmark shapes, the autotuner's choice for a 4096^2 grid, else the configuration's)")
    ap.add_argument("--refine-particles", type=int, default=128)
    ap.add_argument("--no-refine", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--refine-plain-only", action="store_true",
                    help="only time the plain refinement grid on --refine-particles particles (profiling)")
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--no-torch-reference", action="store_true",
                    help="skip timing the reference's torch + cuFFT GPU path on this GPU")
    ap.add_argument("--torch-ref-batches", type=int, default=4)
    ap.add_argument("--torch-ref-streams", type=int, default=4)
    ap.add_argument("--precision-error-orient", type=int, default=10240,
                    help="orientations (uniform random) checked against the FP64 oracle on the small configuration")
    ap.add_argument("--batched-micrographs", type=int, default=12)
    ap.add_argument("--batched-full-grid", type=int, default=-1,
                    help="only time one batched-workload micrograph (this index) over its full grid")
    ap.add_argument("--precision-stage-4096", action="store_true",
                    help="only time one radix-64 DFT-GEMM stage at the 4096^2 production shape")
    ap.add_argument("--learned-eval", type=int, default=0,
                    help="only run learned-proposal refinement on this many simulated particles (e.g. 50000)")
    ap.add_argument("--learned-eval-plain", type=int, default=1024,
                    help="particles of that set also refined by the plain grid for the SNR comparison")
    ap.add_argument("--batched-orient", type=int, default=48,
                    help="orientations searched per micrograph in the batched-form sample")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            ident = str(self.device_index)
            try:
                uuid = str(torch.cuda.get_device_properties(self.device_index).uuid)
                ident = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            except Exception:
                pass
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", ident],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _workload(cfg_name, device):
    from leopard_em_gb300 import synthetic as sy

    cfg = {"production": sy.CONFIG_PRODUCTION, "small": sy.CONFIG_SMALL, "refbench": sy.CONFIG_REFBENCH}[cfg_name]
    return sy.make_match_workload(cfg, device=device)


def _fp32_peak(dev):
    """Non-tensor FP32 peak (TFLOP/s) from the library's FMA probe, best of 3."""
    import ctypes

    from leopard_em_gb300._native import check
    from leopard_em_gb300.build import PROBE_LIB_PATH

    probe = ctypes.CDLL(PROBE_LIB_PATH)
    probe.lgb_fp32_fma_probe.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    probe.lgb_fp32_fma_probe.restype = ctypes.c_int
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = sms * 8, 20000
    out = torch.zeros(1, device=dev)
    stream = torch.cuda.current_stream(dev)
    s = ctypes.c_void_p(stream.cuda_stream)
    flops = blocks * 256 * 8 * 16 * 2.0 * iters
    best = 0.0
    for i in range(4):
        a = torch.cuda.Event(enable_timing=True)
        z = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        check(probe.lgb_fp32_fma_probe(blocks, iters, out.data_ptr(), s), "lgb_fp32_fma_probe")
        z.record(stream)
        z.synchronize()
        if i:
            best = max(best, flops / (a.elapsed_time(z) / 1e3) / 1e12)
    return best


def _cpu_oracle_rate(kwargs, n_orient, batch, threads, start=0):
    """Orientations/s of the CPU oracle on n_orient orientations (bounded sample)."""
    from oracle import ref_match_template as orc

    torch.set_num_threads(threads)
    kw = dict(kwargs)
    kw["euler_angles"] = kwargs["euler_angles"][start : start + n_orient]
    t0 = time.perf_counter()
    orc.core_match_template_cpu(**kw, orientation_batch_size=batch, backend="batched")
    return n_orient / (time.perf_counter() - t0)


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ---------------------------------------------------------------------------
# The reference's own GPU path, torch + cuFFT, timed on this GPU.  Restates the
# operation sequence of Leopard-EM's default ("streamed") search backend:
# do_streamed_orientation_cross_correlate (backend/cross_correlation.py:13-154)
# with round-robin CUDA streams, normalize_template_projection
# (backend/utils.py:106-188) and do_iteration_statistics_updates
# (utils.py:191-255), both torch.compile'd as the reference does (utils.py:259-266;
# eager when compilation fails), inside the orientation loop of
# _core_match_template_single_gpu (backend/core_match_template.py:492-550).
# Central slices (torch-fourier-slice) are a trilinear gather in torch ops.
# ---------------------------------------------------------------------------
def _ref_normalize(projections, small_shape, large_shape):
    top, bottom = projections[..., 0, :], projections[..., -1, :]
    left, right = projections[..., 1:-1, 0], projections[..., 1:-1, -1]
    edge = torch.concatenate([top, bottom, left, right], dim=-1)
    projections = projections - edge.mean(dim=-1)[..., None, None]
    large_sqrt = (large_shape[0] * large_shape[1]) ** 0.5
    rel = (small_shape[0] * small_shape[1]) / (large_shape[0] * large_shape[1])
    mean = torch.mean(projections, dim=(-2, -1), keepdim=True) * rel * rel
    var = torch.sum((projections - mean) ** 2, dim=(-2, -1), keepdim=True)
    var = var + (large_shape[0] - small_shape[0]) * (large_shape[1] - small_shape[1]) * mean**2
    return (projections * large_sqrt) / torch.sqrt(var.clamp_min(1e-8))


def _ref_stats_update(cc, idx, mip, best, s1, s2, h, w):
    ccr = cc.reshape(-1, h, w)
    mv, mi = torch.max(ccr, dim=0)
    upd = mv > mip
    mip.copy_(torch.where(upd, mv, mip))
    best.copy_(torch.where(upd, idx[mi], best))
    s1 += ccr.sum(dim=0)
    s2 += (ccr**2).sum(dim=0)


def _ref_slices(vol, rot):
    """Central slices (B, d, d//2+1) of the fftshifted rfft volume, trilinear,
    Friedel mate for x < 0, zero outside (torch-fourier-slice convention)."""
    d = vol.shape[0]
    dev = vol.device
    fy = torch.fft.fftshift(torch.fft.fftfreq(d, device=dev))
    fx = torch.fft.rfftfreq(d, device=dev)
    gy, gx = torch.meshgrid(fy, fx, indexing="ij")
    zyx = torch.stack([torch.zeros_like(gy), gy, gx], dim=-1)
    r = torch.einsum("bij,hwj->bhwi", torch.flip(rot, dims=(-2, -1)), zyx)
    conj = r[..., 2] < 0
    r = torch.where(conj[..., None], -r, r)
    c = r * d + torch.tensor([d // 2, d // 2, 0.0], device=dev)
    hi = torch.tensor(vol.shape, device=dev, dtype=c.dtype) - 1
    inside = ((c >= 0) & (c <= hi)).all(dim=-1)
    c = torch.minimum(c.clamp_min(0), hi)
    i0 = c.floor().long()
    t = c - i0
    i1 = torch.minimum(i0 + 1, hi.long())
    out = torch.zeros(c.shape[:-1], dtype=vol.dtype, device=dev)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                iz = (i1 if dz else i0)[..., 0]
                iy = (i1 if dy else i0)[..., 1]
                ix = (i1 if dx else i0)[..., 2]
                wgt = ((t[..., 0] if dz else 1 - t[..., 0]) * (t[..., 1] if dy else 1 - t[..., 1])
                       * (t[..., 2] if dx else 1 - t[..., 2]))
                out = out + vol[iz, iy, ix] * wgt
    out = torch.where(inside, out, torch.zeros_like(out))
    return torch.where(conj, out.conj(), out)


def _euler_zyz(e):
    a, b, c = (torch.deg2rad(e[:, i].double()) for i in range(3))

    def rz(t):
        o, z = torch.ones_like(t), torch.zeros_like(t)
        return torch.stack([torch.cos(t), -torch.sin(t), z, torch.sin(t), torch.cos(t), z, z, z, o], -1).view(-1, 3, 3)

    def ry(t):
        o, z = torch.ones_like(t), torch.zeros_like(t)
        return torch.stack([torch.cos(t), z, torch.sin(t), z, o, z, -torch.sin(t), z, torch.cos(t)], -1).view(-1, 3, 3)

    return (rz(a) @ ry(b) @ rz(c)).float()


def torch_cufft_reference(kw, dev, batch, n_batches, n_streams):
    """Orientations/s of the reference's torch + cuFFT GPU path on this GPU
    (same inputs, batch ``batch``, ``n_streams`` CUDA streams), device-timed
    over ``n_batches`` batches after one warm-up batch."""
    image_dft = kw["image_dft"].to(dev)
    template_dft = kw["template_dft"].to(dev)
    pf = (kw["ctf_filters"] * kw["whitening_filter_template"][None, None]).to(dev)
    eul = kw["euler_angles"].to(dev)
    n_cs, n_df = pf.shape[0], pf.shape[1]
    H, W = image_dft.shape[0], 2 * image_dft.shape[1] - 2
    small = (template_dft.shape[1], 2 * template_dft.shape[2] - 2)
    compiled = "inductor (default mode)"
    try:
        norm = torch.compile(_ref_normalize)
        upd = torch.compile(_ref_stats_update)
        norm(torch.randn(2, *small, device=dev), small, (H, W))
    except Exception as e:  # the reference falls back to eager the same way (utils.py:92-100)
        norm, upd, compiled = _ref_normalize, _ref_stats_update, f"eager ({type(e).__name__})"
    streams = [torch.cuda.Stream(dev) for _ in range(n_streams)]
    mip = torch.full((H, W), -float("inf"), device=dev)
    best = torch.full((H, W), -1, dtype=torch.int32, device=dev)
    s1 = torch.zeros((H, W), device=dev)
    s2 = torch.zeros((H, W), device=dev)
    n_o = eul.shape[0]
    incr = torch.tensor([df * n_o + cs * n_df * n_o for cs in range(n_cs) for df in range(n_df)], device=dev)

    def one_batch(o0):
        rot = _euler_zyz(eul[o0:o0 + batch])
        fs = _ref_slices(template_dft, rot)
        fs = torch.fft.ifftshift(fs, dim=(-2,))
        fs[..., 0, 0] = 0
        fs *= -1
        cc = torch.empty((n_cs, n_df, rot.shape[0], H, W), device=dev)
        default = torch.cuda.current_stream(dev)
        for st in streams:
            st.wait_stream(default)
        for i in range(rot.shape[0]):
            for j in range(n_df):
                for k in range(n_cs):
                    st = streams[(i * n_df * n_cs + j * n_cs + k) % n_streams]  # round robin
                    with torch.cuda.stream(st):
                        proj = torch.fft.irfft2(fs[i] * pf[k, j])
                        proj = torch.fft.ifftshift(proj, dim=(-2, -1))
                        proj = norm(proj, small, (H, W))
                        tmp = torch.fft.rfft(proj, n=W, dim=-1)
                        pd = torch.fft.fft(tmp, n=H, dim=-2)
                        pd[0, 0] = 0
                        torch.fft.irfft2(image_dft * pd.conj(), s=(H, W), out=cc[k, j, i])
        for st in streams:
            default.wait_stream(st)
        fs.record_stream(default)
        idx = (torch.arange(o0, o0 + rot.shape[0], device=dev) + incr[:, None]).flatten().to(torch.int32)
        upd(cc, idx, mip, best, s1, s2, H, W)

    one_batch(0)
    torch.cuda.synchronize(dev)
    stream = torch.cuda.current_stream(dev)
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for b in range(n_batches):
        one_batch(((b + 1) * batch) % max(1, n_o - batch))
    z.record(stream)
    torch.cuda.synchronize(dev)
    sec = a.elapsed_time(z) / 1e3
    n = n_batches * batch
    return {"value": n / sec, "unit": UNIT, "cross_correlations_per_s": n * n_cs * n_df / sec,
            "orientations": n, "orientation_batch": batch, "cuda_streams": n_streams, "compiled": compiled,
            "path": "torch.fft (cuFFT) restatement of the reference's streamed GPU backend, same inputs"}


def precision_bench(args, dev):
    """Precision form on the small configuration (512^2 image, 64^3 template,
    grid 20/20 deg = 1,908 orientations): the inverse column and row DFTs as
    split-precision tcgen05 DFT-GEMMs.  Orientations/s of the whole grid for
    the plain FP32 kernels (B = 8 as configured, and B = 32) and the BF16x3 /
    FP16x3 precision forms (B = 32), device-timed; MIP, argmax and z-score
    error of each against an FP64 oracle on the first
    ``--precision-error-orient`` orientations."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300._native import StageProfile
    from leopard_em_gb300.backend import MatchTemplateSearch
    from oracle import ref_match_template as orc

    wl = sy.make_match_workload(sy.CONFIG_SMALL, device=dev)
    kw = wl.kwargs
    N = int(kw["euler_angles"].shape[0])
    H, W = sy.CONFIG_SMALL.image_shape
    d = sy.CONFIG_SMALL.template_size
    stream = torch.cuda.current_stream(dev)
    peaks, _ = _peaks()
    modes = [("fp32_b8", "fp32", 8), ("fp32_b32", "fp32", 32), ("bf16x3_b32", "bf16x3", 32),
             ("fp16x3_b32", "fp16x3", 32)]
    graphs = {"fp32_b8_graph": ("fp32", 8, 32), "fp32_b32_graph": ("fp32", 32, 8)}
    out = {}
    for label, prec, B in modes + [(k, v[0], v[1]) for k, v in graphs.items()]:
        gb = graphs[label][2] if label in graphs else 0
        s = MatchTemplateSearch(**kw, device=dev, orientation_batch_size=B, precision=prec, graph_batches=gb)
        s.run(0, N)  # warm-up: the whole grid once
        reps = 5
        a = torch.cuda.Event(enable_timing=True)
        z = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        a.record(stream)
        for _ in range(reps):
            s.run(0, N)
        z.record(stream)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(z) / reps
        with StageProfile() as prof:
            s.run(0, N)
            torch.cuda.synchronize(dev)
        entry = {"orientations_per_s": N / (ms / 1e3), "ms_per_grid": ms, "orientation_batch": B,
                 "graph_batches": gb,
                 "stage_ms": {k: round(v, 4) for k, v in prof.ms.items() if prof.launches[k]}}
        if prec != "fp32":
            wq = -(-(W // 2 + 1) // 32) * 32
            n_cp = 1 << (B - 1).bit_length()
            flops = {  # useful FLOPs of the three split terms per full batch
                "dft_col_gemm": 2.0 * (2 * H) * (B * wq) * (2 * H) * 3,
                "dft_row_gemm": 2.0 * W * (H * n_cp) * (-(-(2 * (W // 2 + 1)) // 64) * 64) * 3,
            }
            tc = {}
            for k, f in flops.items():
                per = prof.ms[k] / max(1, prof.launches[k])
                tc[k] = {"tflops": f / (per / 1e3) / 1e12, "per_launch_ms": per,
                         "frac_of_bf16_peak": f / (per / 1e3) / 1e12 / peaks.get("bf16_tflops", 1900.0)}
            entry["tensor"] = tc
        out[label] = entry
        del s
    # errors against the FP64 oracle on args.precision_error_orient orientations
    # sampled uniformly from SO(3) (seeded), same image and template; the
    # oracle's torch operations run in FP64 on this GPU
    n_err = max(1, args.precision_error_orient)
    sub = dict(kw)
    sub["euler_angles"] = sy.random_euler_angles(n_err, seed=2024)
    cpu = {k: v.cpu() for k, v in sub.items()}
    t_ref = time.perf_counter()
    ref = orc.core_match_template_cpu(**cpu, orientation_batch_size=32, backend="batched", stat_dtype=torch.float64,
                                      track_second_best=True, compute_dtype=torch.float64, device=dev)
    t_ref = time.perf_counter() - t_ref
    torch.cuda.empty_cache()
    mip_r = ref["mip"].double()
    scale = mip_r.abs().clamp_min(1.0)
    sep = (mip_r - ref["second_best"].double()) > 1e-3 * scale
    for label, prec, B in modes:  # graph replay changes no value: errors as without
        s = MatchTemplateSearch(**sub, device=dev, orientation_batch_size=B, precision=prec)
        s.run()
        res = s.result(to_cpu=True)
        best = s.best_index.cpu().long()
        out[label]["vs_fp64"] = {
            "orientations": n_err, "orientation_sample": "uniform random SO(3), seed 2024",
            "fp64_oracle_s": t_ref,
            "mip_max_rel_err": ((res["mip"].double() - mip_r).abs() / scale).max().item(),
            "argmax_agreement_separated": ((best == ref["best_global_index"].long()) | ~sep).double().mean().item(),
            "argmax_agreement_all": (best == ref["best_global_index"].long()).double().mean().item(),
            "z_max_abs_err": (res["scaled_mip"].double() - ref["scaled_mip"].double()).abs().max().item(),
        }
        del s
    base = out["fp32_b8"]["orientations_per_s"]
    return {"workload": sy.CONFIG_SMALL.name + " (precision form)", "image": [H, W], "template": d,
            "orientations_total": N, "runs": out,
            "speedup_bf16x3_vs_fp32_b8": out["bf16x3_b32"]["orientations_per_s"] / base,
            "speedup_bf16x3_vs_fp32_b32": out["bf16x3_b32"]["orientations_per_s"] / out["fp32_b32"]["orientations_per_s"]}


def batched_bench(args, dev):
    """Batched form: micrographs of uneven sizes (2048^2, 3072x2880, 3838x3710,
    4096^2, 5760x4092 cycled), one 256^3 template, 7 defocus planes x 3 pixel
    sizes, grid 3.0/2.0 deg (825,480 orientations).  Every micrograph searches
    the same ``--batched-orient`` consecutive orientations of the grid (a
    bounded sample of its full search); times are per micrograph, device-timed
    from the upload of its spectrum to its finalised maps.  Run once with the
    autotuned batch / column split and CUDA-graph replay, once with a fixed
    batch of 8 and plain launches."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.backend.batched import match_template_batch

    t0 = time.perf_counter()
    template_dft, eul, mics, cfgs = sy.make_batched_workload(args.batched_micrographs, device=dev)
    gen_s = time.perf_counter() - t0
    N = int(eul.shape[0])
    n = max(1, min(args.batched_orient, N))
    rng = (N // 2, N // 2 + n)
    n_cd = len(sy.CONFIG_BATCHED.defocus_offsets) * len(sy.CONFIG_BATCHED.pixel_size_offsets)
    t0 = time.perf_counter()
    match_template_batch(mics, template_dft, eul, dev, orientation_range=rng, tune=True)  # tune + warm up
    tune_s = time.perf_counter() - t0
    out = {}
    for label, tune, graphs in (("tuned_graph", True, True), ("fixed_b8_plain", False, False)):
        match_template_batch(mics[:1], template_dft, eul, dev, orientation_range=rng, tune=tune, use_graphs=graphs)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        _, rep = match_template_batch(mics, template_dft, eul, dev, orientation_range=rng, tune=tune,
                                      orientation_batch_size=8, use_graphs=graphs)
        wall = time.perf_counter() - t0
        out[label] = {"p50_ms": rep.percentile(50), "p99_ms": rep.percentile(99), "mean_ms": statistics.mean(rep.ms),
                      "per_micrograph_ms": [round(x, 3) for x in rep.ms], "wall_s": wall,
                      "orientations_per_s": len(mics) * n / (sum(rep.ms) / 1e3),
                      "cross_correlations_per_s": len(mics) * n * n_cd / (sum(rep.ms) / 1e3)}
        if tune:
            out[label]["tuning"] = {f"{g[0]}x{g[1]}": {"orientation_batch": t.orientation_batch,
                                                        "col_waves": t.col_waves, "graph_batches": t.graph_batches,
                                                        "transposed": bool(t.transpose)}
                                    for g, t in zip(rep.grids, rep.tunings)}
            out[label]["grids"] = [list(g) for g in rep.grids]
    best = out["tuned_graph"]
    return {
        "workload": sy.CONFIG_BATCHED.name, "micrographs": len(mics),
        "sizes": [list(c.image_shape) for c in cfgs], "particles": [c.n_particles for c in cfgs],
        "snr": [round(c.snr, 4) for c in cfgs], "template": sy.CONFIG_BATCHED.template_size,
        "defocus_planes": len(sy.CONFIG_BATCHED.defocus_offsets),
        "pixel_sizes": len(sy.CONFIG_BATCHED.pixel_size_offsets), "orientations_total": N,
        "orientations_per_micrograph_sample": n, "p50_ms": best["p50_ms"], "p99_ms": best["p99_ms"],
        "full_grid_p50_s_est": best["p50_ms"] / 1e3 * N / n, "full_grid_p99_s_est": best["p99_ms"] / 1e3 * N / n,
        "runs": out, "workload_build_s": gen_s, "tune_and_warmup_s": tune_s,
        "note": "per-micrograph time = spectrum upload + zero-padding + search of the sample + finalize; "
                "full-grid estimates scale the sample linearly",
    }


def batched_full_grid(args):
    """One micrograph of the batched workload (``--batched-full-grid I``: its
    index, 0 = the 2048^2 one) searched over the whole 3.0/2.0-degree grid
    (825,480 orientations x 7 defocus x 3 pixel sizes) through the batched
    driver, autotuned and graph-replayed; device time from the upload of its
    spectrum to its finalised maps.  Not part of the default run (minutes)."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.backend.batched import match_template_batch

    dev = torch.device("cuda", 0)
    i = int(args.batched_full_grid)
    template_dft, eul, mics, cfgs = sy.make_batched_workload(i + 1, device=dev)
    n_cd = len(sy.CONFIG_BATCHED.defocus_offsets) * len(sy.CONFIG_BATCHED.pixel_size_offsets)
    mic = [mics[i]]
    match_template_batch(mic, template_dft, eul, dev, orientation_range=(0, 64), tune=True)  # tune + warm up
    torch.cuda.synchronize(dev)
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        res, rep = match_template_batch(mic, template_dft, eul, dev, tune=True)
        wall = time.perf_counter() - t0
    N = int(eul.shape[0])
    return {"metric": "full-grid search time of one micrograph (batched form)", "value": rep.ms[0] / 1e3,
            "unit": "s", "micrograph": list(cfgs[i].image_shape), "orientations": N, "defocus_x_pixel_sizes": n_cd,
            "cross_correlations": N * n_cd, "cross_correlations_per_s": N * n_cd / (rep.ms[0] / 1e3),
            "wall_s": wall, "grid": list(rep.grids[0]), "tuning": rep.tunings[0].__dict__,
            "clocks": clocks.summary()}


def learned_eval(args):
    """Learned-proposal refinement over a large simulated particle set (the
    refinement configuration's 50,000 crops by default): proposals, small-grid
    verification and full-grid fallback for every particle, and the plain grid
    on a seeded subset of them for the SNR comparison.  Not part of the default
    run (minutes)."""
    from leopard_em_gb300 import proposal as pr
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.backend.core_refine_template import core_refine_template

    dev = torch.device("cuda", 0)
    cfg = sy.CONFIG_REFINE
    n, m = int(args.learned_eval), int(args.learned_eval_plain)
    t0 = time.perf_counter()
    parts = []
    chunk = 4096
    for a in range(0, n, chunk):  # simulated in chunks (independent seeds), one template
        kw_a, _ = sy.make_refine_workload(cfg, min(chunk, n - a), device=dev, seed_offset=50_000 + a)
        parts.append(kw_a)
    kw = dict(parts[0])
    for k, v in parts[0].items():
        if isinstance(v, torch.Tensor) and v.shape[:1] == (min(chunk, n),) and k != "euler_angle_offsets":
            kw[k] = torch.cat([p[k] for p in parts])
    del parts
    t_data = time.perf_counter() - t0
    net = pr.load_net(os.path.join(ROOT, "leopard_em_gb300", "weights", "proposal_refine288.npz"), dev)
    small = sy.local_euler_offsets(0.5, 0.125, 0.5, 0.125)
    small_df = torch.arange(-100.0, 100.0 + 1e-6, 50.0)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    res, info = pr.refine_with_proposals(net, kw, dev, small, small_df, batch_size=cfg.batch)
    torch.cuda.synchronize(dev)
    t_learned = time.perf_counter() - t0
    z = res["refined_z_score"].double()
    sel = torch.randperm(n, generator=torch.Generator().manual_seed(7))[:m].sort().values
    sub = {k: (v[sel] if isinstance(v, torch.Tensor) and v.shape[:1] == (n,) else v) for k, v in kw.items()}
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    plain = core_refine_template(**sub, device=dev, batch_size=cfg.batch)
    torch.cuda.synchronize(dev)
    t_plain = time.perf_counter() - t0
    zp, zl = plain["refined_z_score"].double(), z[sel]
    return {"metric": "learned-proposal refinement over a large simulated particle set",
            "workload": cfg.name, "particles": n, "data_seconds": t_data,
            "learned": {"value": n / t_learned, "unit": "particles/s", "seconds": t_learned,
                        "fallbacks": info["fallback"], "fallback_rate": info["fallback"] / n,
                        "correlations_per_particle": info["correlations_per_particle"],
                        "mean_refined_snr": float(z.mean())},
            "plain_subset": {"particles": m, "value": m / t_plain, "unit": "particles/s",
                             "mean_refined_snr": float(zp.mean()), "learned_mean_refined_snr": float(zl.mean()),
                             "learned_at_least_plain": bool(zl.mean() >= zp.mean()),
                             "particles_below_plain": int((zl < zp - 1e-6).sum())},
            "timing": "wall clock, host tensors in and out"}


def precision_stage_4096(args):
    """One radix-64 DFT-GEMM stage of a factored inverse column transform at
    the production shape (48 correlograms x 2,049 columns x 64 = 6.29 M rows,
    K = N = 128 real values = 64 complex points in and out) on the tcgen05
    GEMM, with one and three BF16 terms: the measured floor of a 4096^2
    precision form.  Not part of the default run."""
    import ctypes

    from leopard_em_gb300 import precision as pc
    from leopard_em_gb300._native import check, lib

    dev = torch.device("cuda", 0)
    M, K, N = 48 * 2049 * 64, 128, 128
    g = torch.Generator(device=dev).manual_seed(0)
    a = torch.randn(M, K, device=dev, generator=g)
    b = torch.randn(N, K, device=dev, generator=g)
    a_hi, a_lo = pc.blocked_split(a, 128)
    b_hi, b_lo = pc.blocked_split(b, 128)
    del a
    d = torch.empty((M, N), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    out = {"metric": "one radix-64 DFT-GEMM stage at the 4096^2 production shape", "M": M, "N": N, "K": K}
    for terms in (3, 1):
        def run():
            check(lib().lgb_tc_gemm(M // 128, 1, K // 64, 128, 0, terms, a_hi.data_ptr(), a_lo.data_ptr(),
                                    b_hi.data_ptr(), b_lo.data_ptr(), d.data_ptr(), N, M, N, err.data_ptr(), s),
                  "lgb_tc_gemm")

        for _ in range(2):
            run()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record()
        for _ in range(5):
            run()
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / 5
        out[f"bf16x{terms}"] = {"ms": ms, "tflops": 2 * M * N * K * terms / (ms / 1e3) / 1e12,
                                "operand_gb": M * K * 2 * (2 if terms == 3 else 1) / 1e9, "output_gb": M * N * 4 / 1e9}
    if int(err.item()):
        raise RuntimeError("lgb_tc_gemm: device status %d" % int(err.item()))
    return out


def refine_plain_only(args):
    """Plain refinement grid alone (device-timed particles/s), for profiling."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.backend.core_refine_template import refine_particles_device

    dev = torch.device("cuda", 0)
    cfg = sy.CONFIG_REFINE
    n = args.refine_particles
    kw, _ = sy.make_refine_workload(cfg, n, device=dev)
    dkw = {k: (v.to(dev) if isinstance(v, torch.Tensor) else v) for k, v in kw.items()}
    warm = dict(dkw)
    warm["euler_angle_offsets"] = dkw["euler_angle_offsets"][: 2 * cfg.batch]
    refine_particles_device(**warm, device=dev, batch_size=cfg.batch)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    refine_particles_device(**dkw, device=dev, batch_size=cfg.batch)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    out = {"metric": "refined particles/s (plain local grid)", "value": n / (e0.elapsed_time(e1) / 1e3),
           "unit": "particles/s", "particles": n, "workload": cfg.name}
    # a second, separately timed pass with the per-stage events on
    from leopard_em_gb300._native import StageProfile

    with StageProfile() as prof:
        refine_particles_device(**dkw, device=dev, batch_size=cfg.batch)
        torch.cuda.synchronize(dev)
    out["stage_ms_per_launch"] = {k: round(prof.ms[k] / prof.launches[k], 4) for k in prof.ms if prof.launches[k]}
    return out


def refine_bench(args, dev, with_cpu):
    """Refined particles/s of the plain local grid (288^2 crops, 256^3 template,
    +-3 deg @ 0.25 deg x +-400 A @ 50 A)."""
    from leopard_em_gb300 import synthetic as sy
    from leopard_em_gb300.backend import core_refine_template
    from leopard_em_gb300.backend.core_refine_template import refine_particles_device

    cfg = sy.CONFIG_REFINE
    n = args.refine_particles
    kw, _ = sy.make_refine_workload(cfg, n, device=dev)
    dkw = {k: (v.to(dev) if isinstance(v, torch.Tensor) else v) for k, v in kw.items()}
    warm = dict(dkw)
    warm["euler_angle_offsets"] = dkw["euler_angle_offsets"][: 2 * cfg.batch]
    refine_particles_device(**warm, device=dev, batch_size=cfg.batch)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    raw = refine_particles_device(**dkw, device=dev, batch_size=cfg.batch)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    dev_s = e0.elapsed_time(e1) / 1e3
    t0 = time.perf_counter()
    res = core_refine_template(**kw, device=dev, batch_size=cfg.batch)
    e2e_s = time.perf_counter() - t0
    K = int(kw["euler_angle_offsets"].shape[0])
    D = int(kw["defocus_offsets"].shape[0])
    out = {
        "metric": "refined particles/s (plain local grid)", "value": n / dev_s, "unit": "particles/s",
        "e2e": n / e2e_s, "particles": n, "offsets": K, "defocus": D,
        "cross_correlations_per_particle": K * D, "cross_correlations_per_s": n * K * D / dev_s,
        "mean_refined_snr": float(res["refined_z_score"].mean()),
        "workload": cfg.name,
    }
    lr = learned_refine_bench(kw, dev, cfg, res, n)
    out.update(lr)
    if lr.get("learned"):
        out["learned_speedup_vs_plain_e2e"] = lr["learned"]["value"] / out["e2e"]
    if with_cpu:
        from oracle import ref_refine_template as orr

        m = 16
        ck = {k: v for k, v in kw.items()}
        ck["euler_angle_offsets"] = kw["euler_angle_offsets"][:m]
        sub = {k: (v[:1] if isinstance(v, torch.Tensor) and v.shape[0] == n else v) for k, v in ck.items()}
        torch.set_num_threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        orr.core_refine_template_cpu(**sub, batch_size=m)
        cpu_s = (time.perf_counter() - t0) * K / m
        out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "particles/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": f"1 particle x {m} offsets x {D} defocus, extrapolated to {K} offsets"}
    return out


def network_timing(dev, infer_batch=1024, train_batch=256, reps=5):
    """Proposal-network time per particle through the tensor-core kernels:
    inference (forward at ``infer_batch``) and one training step (forward,
    backward, Adam at ``train_batch``), CUDA events on the current stream."""
    from leopard_em_gb300 import proposal as pr

    net = pr.ProposalNet(dev, seed=0)
    g = torch.Generator().manual_seed(5)
    x = torch.randn(infer_batch, pr.CHANNELS, pr.BAND, pr.BAND, generator=g).to(dev, torch.bfloat16)
    tgt = torch.randn(train_batch, 7, generator=g).to(dev)
    flops = 0  # multiply-adds x 2 per sample, forward
    hw = pr.BAND
    for kind, cin, cout, stride, _ in pr.LAYERS:
        if kind == "conv":
            hw = (hw - 1) // stride + 1
            flops += 2 * hw * hw * cout * cin * 9
        else:
            flops += 2 * cin * cout

    def train_step():
        out = net.forward(x[:train_batch])
        _, dout = net.loss_and_grad(out, tgt)
        net.backward(dout)
        net.adam_step(1e-4)

    res = {}
    for label, fn, n in (("inference", lambda: net.forward(x), infer_batch), ("train_step", train_step, train_batch)):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize(dev)
        sec = e0.elapsed_time(e1) / 1e3 / reps
        mult = 1 if label == "inference" else 3  # backward ~ 2x forward
        res[label] = {"us_per_particle": 1e6 * sec / n, "batch": n, "ms_per_batch": 1e3 * sec,
                      "tflops": mult * flops * n / sec / 1e12}
    net.check_device_status()
    res["forward_mflop_per_particle"] = flops / 1e6
    res["kernels"] = "conv3x3 (implicit GEMM) and linear layers on tcgen05: BF16 operands, FP32 TMEM accumulation"
    return res


def learned_refine_bench(kw, dev, cfg, plain_res, n_plain):
    """Learned proposals + small local grid (fallback: full plain grid) on the
    same particles as the plain grid, and the Gauss-Newton-only ablation (the
    network's input channels' linearised step, no network) through the same
    verification and fallback.  Wall-clock particles/s with host tensors in and
    out, like the plain grid's ``e2e``."""
    from leopard_em_gb300 import proposal as pr
    from leopard_em_gb300 import synthetic as sy

    path = os.path.join(ROOT, "leopard_em_gb300", "weights", "proposal_refine288.npz")
    if not os.path.exists(path):
        return {"learned": None}
    net = pr.load_net(path, dev)
    # +-0.5 deg at 0.125 deg: the same 576 offsets as +-1 deg at 0.25 deg, finer
    # (the proposals are within ~0.2 deg)
    small = sy.local_euler_offsets(0.5, 0.125, 0.5, 0.125)
    small_df = torch.arange(-100.0, 100.0 + 1e-6, 50.0)
    warm = {k: (v[:4] if isinstance(v, torch.Tensor) and v.shape[:1] == (n_plain,) else v) for k, v in kw.items()}
    pr.refine_with_proposals(net, warm, dev, small, small_df, batch_size=cfg.batch)
    zp = plain_res["refined_z_score"].double()
    out = {}
    for label, which in (("learned", "network"), ("gauss_newton_only", "gauss_newton")):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        res, info = pr.refine_with_proposals(net if which == "network" else None, kw, dev, small, small_df,
                                             batch_size=cfg.batch, proposal=which)
        torch.cuda.synchronize(dev)
        dt = time.perf_counter() - t0
        z = res["refined_z_score"].double()
        out[label] = {"metric": "refined particles/s (proposal + local grid, full-grid fallback)",
                      "proposal": which, "value": n_plain / dt, "unit": "particles/s", "particles": n_plain,
                      "fallbacks": info["fallback"], "fallback_rate": info["fallback"] / n_plain,
                      "correlations_per_particle": info["correlations_per_particle"],
                      "mean_refined_snr": float(z.mean()), "plain_mean_refined_snr": float(zp.mean()),
                      "snr_at_least_plain": bool(z.mean() >= zp.mean()),
                      "particles_below_plain": int((z < zp - 1e-6).sum()),
                      "small_grid": "+-0.5 deg @ 0.125 x +-100 A @ 50",
                      "timing": "wall clock, host tensors in and out (network inputs, inference, two refinement "
                                "calls and any fallback)"}
    out["network_timing"] = network_timing(dev)
    return out


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return
    from leopard_em_gb300 import synthetic as sy

    cfg = {"production": sy.CONFIG_PRODUCTION, "small": sy.CONFIG_SMALL, "refbench": sy.CONFIG_REFBENCH}[args.config]
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    wl = sy.make_match_workload(cfg, device=dev)
    cpu_kw = {k: (v.cpu() if isinstance(v, torch.Tensor) else v) for k, v in wl.kwargs.items()}  # host copies, once
    threads = os.cpu_count() or 1
    per_step = 1 if args.config in ("production", "refbench") else 8
    # the orientation batch our arm reports for this workload (the CPU oracle's
    # correlograms do not depend on it)
    B = args.batch if args.batch > 0 else cfg.orientation_batch
    if args.batch < 0 and args.config in ("production", "refbench"):
        B = 64
    for i in range(args.warmup):
        _cpu_oracle_rate(cpu_kw, per_step, cfg.orientation_batch, threads, start=i * per_step)
    t0 = time.perf_counter()
    for i in range(args.steps):
        _cpu_oracle_rate(cpu_kw, per_step, cfg.orientation_batch, threads, start=(args.warmup + i) * per_step)
    dt = time.perf_counter() - t0
    value = args.steps * per_step / dt
    sample = (f"{per_step} orientation(s) x {len(cfg.defocus_offsets)} defocus per step of the {cfg.name} "
              f"workload, CPU oracle (torch.fft/pocketfft restatement of the reference's CPU path)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": cfg.name, "image": list(cfg.image_shape), "template": cfg.template_size,
                   "defocus_planes": len(cfg.defocus_offsets), "orientation_batch": B},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    args = _args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.precision_stage_4096:
        print(json.dumps(precision_stage_4096(args)), flush=True)
        return
    if args.learned_eval > 0:
        print(json.dumps(learned_eval(args)), flush=True)
        return
    if args.refine_plain_only:
        print(json.dumps(refine_plain_only(args)), flush=True)
        return
    if args.batched_full_grid >= 0:
        print(json.dumps(batched_full_grid(args)), flush=True)
        return
    rank, world, local = _dist()
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from leopard_em_gb300._native import StageProfile
    from leopard_em_gb300.backend import MatchTemplateSearch, core_match_template

    wl = _workload(args.config, dev)
    cfg = wl.config
    kw = wl.kwargs
    N = kw["euler_angles"].shape[0]
    B = args.batch if args.batch > 0 else cfg.orientation_batch
    if args.batch < 0 and args.config in ("production", "refbench"):
        B = 64
    chunk = max(B, (args.orient_per_step // B) * B)
    search = MatchTemplateSearch(**kw, device=dev, orientation_batch_size=B)
    stream = torch.cuda.current_stream(dev)

    def chunk_range(step):
        first = ((step * world + rank) * chunk) % max(1, N - chunk)
        return first, first + chunk

    for i in range(args.warmup):
        search.run(*chunk_range(i))
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        with StageProfile() as prof:
            torch.cuda.synchronize(dev)
            ev0.record(stream)
            for i in range(args.steps):
                search.run(*chunk_range(args.warmup + i))
            ev1.record(stream)
            torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * args.steps * chunk / (ms / 1e3)

    # --- roofline of the dominant kernel -------------------------------------
    H, W = cfg.image_shape
    d = cfg.template_size
    n_cd = len(cfg.defocus_offsets) * len(cfg.pixel_size_offsets)
    n_c = n_cd * B
    wc = W // 2 + 1
    alg_bytes = {
        "colpass": 8.0 * (n_c * d * wc + H * wc + n_c * H * wc),
        "rowpass": 8.0 * n_c * H * wc + 2.0 * H * W * (4 + 4 + 8 + 8),
        "pad_rfft": 4.0 * n_c * d * d + 8.0 * n_c * d * wc,
    }
    alg_flops = {
        "colpass": n_c * wc * 2 * 5.0 * H * math.log2(H),
        "rowpass": n_c * H * 2.5 * W * math.log2(W),
        "pad_rfft": n_c * d * 2.5 * W * math.log2(W),
    }
    stage_ms, launches = prof.ms, prof.launches
    fp32_peak = None  # measured after the end-to-end calls (its FMA loop runs the GPU at full power)
    top = max(stage_ms, key=stage_ms.get)
    peaks, peak_kind = _peaks()
    per_launch_ms = stage_ms[top] / max(1, launches[top])
    ach = alg_bytes.get(top, 0.0) / (per_launch_ms / 1e3) / 1e9 if top in alg_bytes else None
    # DRAM bytes (read + write) of one launch, from ncu captures of this
    # workload (dram__bytes_read.sum + dram__bytes_write.sum; one launch each,
    # --set full) at orientation batch 8, 16 and 32.  Batch 64 holds too much
    # device memory for a multi-pass capture: its figures extend the 16 and 32
    # captures linearly in the correlograms per launch (colpass 3.657 -> 7.357
    # GB for 48 -> 96; rowpass 4.042 -> 7.282 GB, of which 0.80 GB is the map
    # read-modify-write that does not grow).
    measured_traffic = {("production", 8, "colpass"): 1.875e9, ("production", 8, "rowpass"): 2.390e9,
                        ("production", 16, "colpass"): 3.657e9, ("production", 16, "rowpass"): 4.042e9,
                        ("production", 32, "colpass"): 7.357e9, ("production", 32, "rowpass"): 7.282e9,
                        ("production", 64, "colpass"): 14.757e9, ("production", 64, "rowpass"): 13.762e9}
    roofline = {
        "bound": "hbm", "kernel": top, "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": (ach / peaks["hbm_gbs"]) if ach else None,
        "traffic": measured_traffic.get((args.config, B, top)), "algorithmic_bytes": alg_bytes.get(top),
        "peak_source": peak_kind,
        "per_launch_ms": per_launch_ms,
        "fp32_tflops_achieved": (alg_flops[top] / (per_launch_ms / 1e3) / 1e12) if top in alg_flops else None,
        "fp32_peak_tflops_measured": fp32_peak,
        "stage_share": {k: v / max(1e-9, sum(stage_ms.values())) for k, v in stage_ms.items()},
    }
    gpu_launches = int(sum(launches.values()))

    # --- end to end through the public API with host buffers ------------------
    host = {}
    for k, v in kw.items():
        host[k] = v.pin_memory() if v.device.type == "cpu" else v.cpu().pin_memory()
    e2e_chunk = max(B, (args.e2e_orient // B) * B)

    def e2e_range(step):
        first = ((step * world + rank) * e2e_chunk) % max(1, N - e2e_chunk)
        return first, first + e2e_chunk

    h2d = sum(v.numel() * v.element_size() for k, v in host.items() if k != "euler_angles") + e2e_chunk * 3 * 4
    e2e_times = []
    d2h = 0
    for i in range(args.warmup + args.e2e_steps if args.e2e_steps > 0 else 0):
        a, b = e2e_range(i)
        kw_i = dict(host)
        kw_i["euler_angles"] = host["euler_angles"][a:b]
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        res = core_match_template(**kw_i, device=dev, orientation_batch_size=B)
        torch.cuda.synchronize(dev)
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
        d2h = sum(v.numel() * v.element_size() for v in res.values() if isinstance(v, torch.Tensor))
    e2e_val = e2e_chunk / statistics.median(e2e_times) * world if e2e_times else None
    # the reference benchmark's two-run model T = N / r + k (benchmark_match_template.py:84-123):
    # calls of N/2 and N orientations give the rate r without the per-call set-up k
    two_run = None
    if e2e_times:
        half = max(B, (e2e_chunk // 2 // B) * B)
        t_half = []
        for i in range(max(2, args.e2e_steps)):
            a, _ = e2e_range(i)
            kw_i = dict(host)
            kw_i["euler_angles"] = host["euler_angles"][a:a + half]
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            core_match_template(**kw_i, device=dev, orientation_batch_size=B)
            torch.cuda.synchronize(dev)
            t_half.append(time.perf_counter() - t0)
        t1, t2 = statistics.median(t_half), statistics.median(e2e_times)
        if t2 > t1:
            r = (e2e_chunk - half) / (t2 - t1)
            two_run = {"rate": r * world, "setup_s": t1 - half / r, "n1": half, "n2": e2e_chunk}

    roofline["fp32_peak_tflops_measured"] = _fp32_peak(dev)

    # --- CPU baseline (rank 0, N=1 only) ---------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n = args.cpu_sample_orient if args.config == "production" else 64
        cpu_kw = {k: v.cpu() for k, v in kw.items()}
        rate = _cpu_oracle_rate(cpu_kw, n, B if n % B == 0 else 1, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} orientations x {n_cd} defocus of the {cfg.name} workload, CPU oracle "
                         "(torch.fft/pocketfft restatement of the reference's CPU path)"}

    torch_ref = None
    if rank == 0 and world == 1 and not args.no_torch_reference:
        torch_ref = torch_cufft_reference(kw, dev, B, args.torch_ref_batches, args.torch_ref_streams)
        torch_ref["value_over_torch_cufft"] = value / torch_ref["value"]
        if e2e_val:
            torch_ref["e2e_over_torch_cufft"] = e2e_val / torch_ref["value"]

    refine = None
    if rank == 0 and world == 1 and not args.no_refine:
        refine = refine_bench(args, dev, with_cpu=not args.no_cpu_baseline)

    batched = None
    if rank == 0 and world == 1 and not args.no_batched:
        batched = batched_bench(args, dev)
    precision = None
    if rank == 0 and world == 1 and not args.no_precision:
        precision = precision_bench(args, dev)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian-blob template, N(0,1) image)",
            "config": {"workload": cfg.name, "image": [H, W], "template": d, "defocus_planes": n_cd,
                       "orientation_batch": B, "orientations_per_step": chunk, "orientations_total": N,
                       "cross_correlations_per_s": value * n_cd,
                       "l2": f"inputs larger than L2 ({8 * n_cd * B * H * (W // 2 + 1) / 1e9:.1f} GB correlogram "
                             "intermediate per batch)",
                       "parallelism": f"orientation-sharded x{world}"},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "orientations_per_call": e2e_chunk, "two_run_model": two_run,
                    "call_ms": [round(1e3 * t, 2) for t in e2e_times],
                    "timing": "wall clock per core_match_template call on pinned host tensors: upload, search, "
                              "finalize, all maps back to the host"},
            "roofline": roofline, "cpu_baseline": cpu, "gpu_torch_baseline": torch_ref,
            "gpu_launches": gpu_launches,
            "clocks": clocks.summary(),
            "refine": refine,
            "batched": batched,
            "precision": precision,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
