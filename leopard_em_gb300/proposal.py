"""Learned orientation / defocus proposals for the local refinement.

A BF16 CNN (5 conv + 3 linear layers, 3.11 M parameters) sees, per particle,
the low-frequency band of its spectrum (shift-aligned to the reference), the
template's central slice at its starting pose on the same band, and that
reference's derivatives for small rotations about the three image axes and
for defocus (``lgb_nn_make_inputs``) -- the inputs of a Gauss-Newton step,
which the network learns -- and predicts the
rotation that takes the starting pose to the particle's pose (6D
representation: the first two columns of the delta rotation, applied on the
left like the refinement offsets) and the defocus offset.  Every layer's
forward and backward pass runs on the tcgen05 tensor cores (``csrc/nn_tc.cu``),
the Adam update and the input builder are this package's CUDA kernels
(``csrc/nn.cu``); torch only holds device memory.

The network is trained only on particles produced by the method's own
simulator (``synthetic.simulate_particles``).  Refinement with proposals
(``refine_with_proposals``) runs the plain local grid twice on a small
neighbourhood -- around the proposal and around the starting pose -- and falls
back to the full plain grid for particles whose proposal does not score higher
than the neighbourhood of the starting pose.
"""

from __future__ import annotations

import ctypes
import json
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import rotations as rot
from ._native import CtfParams, check, lib

BAND = 64
IMAGE_CHANNELS = 6  # particle, reference, d/d(rot x, y, z), d/d(defocus)
CHANNELS = 12       # + constant maps of the Gauss-Newton step (shift x, y, rot x, y, z, defocus)
# (kind, in, out, stride, relu); conv input spatial sizes 64 -> 32 -> 16 -> 8 -> 4 -> 4
LAYERS = [
    ("conv", CHANNELS, 48, 2, True),
    ("conv", 48, 96, 2, True),
    ("conv", 96, 128, 2, True),
    ("conv", 128, 128, 2, True),
    ("conv", 128, 128, 1, True),
    ("fc", 128 * 4 * 4, 1152, 1, True),
    ("fc", 1152, 256, 1, True),
    ("fc", 256, 7, 1, False),
]
ROT_SCALE = math.radians(3.0)  # 6D-delta targets are (col - identity) / ROT_SCALE
DEFOCUS_SCALE = 400.0          # defocus-offset target in units of 400 A


def _check_layers(layers) -> None:
    """Convolutions first (BAND x BAND input, CHANNELS channels, <= 128
    channels each), then linear layers; the first linear layer takes the
    flattened last feature map; the last layer has 7 outputs."""
    hw, ch, seen_fc = BAND, CHANNELS, False
    for kind, cin, cout, stride, _ in layers:
        if kind == "conv":
            if seen_fc or cin != ch or not 1 <= cout <= 128 or stride not in (1, 2):
                raise ValueError(f"bad convolution layer {(kind, cin, cout, stride)}")
            hw, ch = (hw - 1) // stride + 1, cout
        elif kind == "fc":
            if cin != (ch * hw * hw if not seen_fc else ch):
                raise ValueError(f"linear layer input {cin} does not match the previous layer's {ch}x{hw}x{hw}")
            seen_fc, ch, hw = True, cout, 1
        else:
            raise ValueError(f"unknown layer kind {kind!r}")
    if ch != 7:
        raise ValueError("the last layer must have 7 outputs")


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _p(t):
    return t.data_ptr() if t is not None else None


class ProposalNet:
    """Parameters, activations and optimizer state of the proposal CNN."""

    def __init__(self, device, seed: int = 0, layers=None):
        self.dev = torch.device(device)
        self.layers = [tuple(l) for l in (layers if layers is not None else LAYERS)]
        _check_layers(self.layers)
        g = torch.Generator().manual_seed(seed)
        self.w, self.b = [], []
        for kind, cin, cout, _, _ in self.layers:
            fan_in = cin * 9 if kind == "conv" else cin
            shape = (cout, cin, 3, 3) if kind == "conv" else (cout, cin)
            self.w.append((torch.randn(shape, generator=g) * math.sqrt(2.0 / fan_in)).to(self.dev))
            self.b.append(torch.zeros(cout, device=self.dev))
        self.w[-1].mul_(0.1)
        self.wbf = [w.to(torch.bfloat16) for w in self.w]
        self.gw = [torch.zeros_like(w) for w in self.w]
        self.gb = [torch.zeros_like(b) for b in self.b]
        self.mw = [torch.zeros_like(w) for w in self.w]
        self.vw = [torch.zeros_like(w) for w in self.w]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.step_count = 0
        self._ws = torch.empty(0, dtype=torch.uint8, device=self.dev)
        self.device_status = torch.zeros(1, dtype=torch.int32, device=self.dev)

    def _workspace(self, N: int, kind: str, cin: int, hw: int, cout: int, stride: int) -> torch.Tensor:
        """Operand workspace of the tensor-core layers, grown to the largest layer seen."""
        need = ctypes.c_size_t(0)
        if kind == "conv":
            check(lib().lgb_nn_conv3x3_workspace_size(N, cin, hw, hw, cout, stride, ctypes.byref(need)),
                  "conv workspace")
        else:
            check(lib().lgb_nn_linear_workspace_size(N, cin, cout, ctypes.byref(need)), "linear workspace")
        if self._ws.numel() < need.value:
            self._ws = torch.empty(need.value, dtype=torch.uint8, device=self.dev)
        return self._ws

    def check_device_status(self) -> None:
        """Raise if a bounded device wait of the tensor-core kernels ran out (synchronises)."""
        st = int(self.device_status.item())
        if st:
            check(st, "proposal network kernels")

    @property
    def n_params(self) -> int:
        return sum(w.numel() + b.numel() for w, b in zip(self.w, self.b))

    # ---- forward / backward through the CUDA kernels --------------------------
    def forward(self, x: torch.Tensor):
        """x: bf16 (N, 6, 64, 64) on the device -> f32 (N, 7); keeps activations."""
        L = lib()
        s = _stream(self.dev)
        N = x.shape[0]
        acts = [x.contiguous()]
        hw = BAND
        out = None
        for i, (kind, cin, cout, stride, relu) in enumerate(self.layers):
            a = acts[-1]
            if kind == "conv":
                ho = (hw - 1) // stride + 1
                y = torch.empty((N, cout, ho, ho), dtype=torch.bfloat16, device=self.dev)
                ws = self._workspace(N, kind, cin, hw, cout, stride)
                check(L.lgb_nn_conv3x3_forward(N, cin, hw, hw, cout, stride, int(relu), _p(a), _p(self.wbf[i]),
                                               _p(self.b[i]), _p(y), _p(ws), ws.numel(), _p(self.device_status), s),
                      "conv forward")
                hw = ho
                acts.append(y)
            else:
                last = i == len(self.layers) - 1
                ybf = torch.empty((N, cout), dtype=torch.bfloat16, device=self.dev)
                yf = torch.empty((N, cout), dtype=torch.float32, device=self.dev) if last else None
                ws = self._workspace(N, kind, cin, 1, cout, 1)
                check(L.lgb_nn_linear_forward(N, cin, cout, int(relu), _p(a), _p(self.wbf[i]), _p(self.b[i]),
                                              _p(ybf), _p(yf), _p(ws), ws.numel(), _p(self.device_status), s),
                      "linear forward")
                acts.append(ybf)
                out = yf
        self._acts = acts
        return out

    def backward(self, dout: torch.Tensor) -> None:
        """dout: f32 (N, 7) = dLoss/dOutput; fills self.gw / self.gb."""
        L = lib()
        s = _stream(self.dev)
        acts = self._acts
        N = dout.shape[0]
        g = dout.contiguous()
        sizes = [BAND]
        for kind, _, _, stride, _ in self.layers:
            if kind == "conv":
                sizes.append((sizes[-1] - 1) // stride + 1)
        for i in range(len(self.layers) - 1, -1, -1):
            kind, cin, cout, stride, relu = self.layers[i]
            if relu:
                gg = torch.empty_like(g)
                check(L.lgb_nn_relu_backward(g.numel(), _p(acts[i + 1]), _p(g), _p(gg), s), "relu backward")
                g = gg
            x = acts[i]
            need_dx = i > 0
            if kind == "fc":
                dx = torch.empty((N, cin), dtype=torch.float32, device=self.dev) if need_dx else None
                ws = self._workspace(N, kind, cin, 1, cout, 1)
                check(L.lgb_nn_linear_backward(N, cin, cout, _p(x), _p(self.wbf[i]), _p(g), _p(dx), _p(self.gw[i]),
                                               _p(self.gb[i]), _p(ws), ws.numel(), _p(self.device_status), s),
                      "linear backward")
            else:
                hw = sizes[i]
                dx = torch.empty((N, cin, hw, hw), dtype=torch.float32, device=self.dev) if need_dx else None
                ws = self._workspace(N, kind, cin, hw, cout, stride)
                check(L.lgb_nn_conv3x3_backward(N, cin, hw, hw, cout, stride, _p(x), _p(self.wbf[i]), _p(g), _p(dx),
                                                _p(self.gw[i]), _p(self.gb[i]), _p(ws), ws.numel(),
                                                _p(self.device_status), s), "conv backward")
            if need_dx:
                g = dx.reshape(acts[i].shape) if self.layers[i - 1][0] == "conv" and kind == "fc" else dx

    def adam_step(self, lr: float, weight_decay: float = 0.0) -> None:
        L = lib()
        s = _stream(self.dev)
        self.step_count += 1
        for i in range(len(self.layers)):
            check(L.lgb_nn_adam(self.w[i].numel(), _p(self.w[i]), _p(self.gw[i]), _p(self.mw[i]), _p(self.vw[i]),
                                _p(self.wbf[i]), lr, 0.9, 0.999, 1e-8, weight_decay, self.step_count, s), "adam w")
            check(L.lgb_nn_adam(self.b[i].numel(), _p(self.b[i]), _p(self.gb[i]), _p(self.mb[i]), _p(self.vb[i]),
                                None, lr, 0.9, 0.999, 1e-8, 0.0, self.step_count, s), "adam b")

    def loss_and_grad(self, out: torch.Tensor, target: torch.Tensor):
        L = lib()
        dout = torch.empty_like(out)
        loss = torch.empty(1, device=self.dev)
        check(L.lgb_nn_mse(out.shape[0], out.shape[1], _p(out), _p(target.contiguous()), None, _p(dout), _p(loss),
                           _stream(self.dev)), "mse")
        return loss, dout

    # ---- persistence ------------------------------------------------------------
    def state(self) -> dict:
        return {f"w{i}": w.cpu().numpy() for i, w in enumerate(self.w)} | {
            f"b{i}": b.cpu().numpy() for i, b in enumerate(self.b)}

    def load(self, state: dict) -> None:
        for i in range(len(self.layers)):
            if tuple(state[f"w{i}"].shape) != tuple(self.w[i].shape):
                raise ValueError(f"layer {i}: stored weights {tuple(state[f'w{i}'].shape)} do not fit "
                                 f"{tuple(self.w[i].shape)}")
            self.w[i].copy_(torch.from_numpy(np.asarray(state[f"w{i}"])).to(self.dev))
            self.b[i].copy_(torch.from_numpy(np.asarray(state[f"b{i}"])).to(self.dev))
            self.wbf[i] = self.w[i].to(torch.bfloat16)


# ---- inputs and targets ---------------------------------------------------------
def make_inputs(particle_dft, template_dft, rotations, defocus_u, defocus_v, defocus_angle, ctf: CtfParams, device):
    """Network inputs bf16 (P, 12, 64, 64) and the Gauss-Newton step f32 (P, 8)
    (see lgb_nn_make_inputs / lgb_nn_gauss_newton)."""
    dev = torch.device(device)
    P, H, wc = particle_dft.shape
    out = torch.empty((P, CHANNELS, BAND, BAND), dtype=torch.bfloat16, device=dev)
    gn = torch.empty((P, 8), dtype=torch.float32, device=dev)
    f32 = dict(device=dev, dtype=torch.float32)
    args = [particle_dft.to(dev, torch.complex64).contiguous(), template_dft.to(dev, torch.complex64).contiguous(),
            rotations.to(**f32).contiguous().reshape(P, 9), defocus_u.to(**f32).contiguous(),
            defocus_v.to(**f32).contiguous(), defocus_angle.to(**f32).contiguous()]
    check(lib().lgb_nn_make_inputs(P, H, 2 * (wc - 1), _p(args[0]), _p(args[1]), template_dft.shape[0], _p(args[2]),
                                   _p(args[3]), _p(args[4]), _p(args[5]), ctypes.byref(ctf), BAND, CHANNELS,
                                   _p(out), _stream(dev)), "make inputs")
    check(lib().lgb_nn_gauss_newton(P, BAND, CHANNELS, _p(out), _p(gn), _stream(dev)), "gauss-newton")
    return out, gn


def rotvec_to_rotmat(w_deg: torch.Tensor) -> torch.Tensor:
    """(N, 3) rotation vectors in degrees -> (N, 3, 3) (Rodrigues), float64."""
    w = torch.deg2rad(w_deg.double())
    th = w.norm(dim=1).clamp_min(1e-12)
    k = w / th[:, None]
    K = torch.zeros(w.shape[0], 3, 3, dtype=torch.float64, device=w.device)
    K[:, 0, 1], K[:, 0, 2], K[:, 1, 0] = -k[:, 2], k[:, 1], k[:, 2]
    K[:, 1, 2], K[:, 2, 0], K[:, 2, 1] = -k[:, 0], -k[:, 1], k[:, 0]
    s, c = th.sin()[:, None, None], th.cos()[:, None, None]
    return torch.eye(3, dtype=torch.float64, device=w.device) + s * K + (1 - c) * (K @ K)


def gauss_newton_proposal(gn: torch.Tensor):
    """The linearised step alone: (delta rotation (N,3,3), defocus offset (N,) A)."""
    return rotvec_to_rotmat(gn[:, 2:5].cpu()), gn[:, 5].cpu().double() * 100.0


def targets_from(r_true: torch.Tensor, r_start: torch.Tensor, ddf: torch.Tensor) -> torch.Tensor:
    """(N, 7): (first two columns of R_true R_start^T - identity) / ROT_SCALE, ddf / DEFOCUS_SCALE."""
    delta = r_true.double() @ r_start.double().transpose(-1, -2)
    eye = torch.eye(3, dtype=torch.float64, device=delta.device)
    six = torch.cat([delta[:, :, 0] - eye[:, 0], delta[:, :, 1] - eye[:, 1]], dim=1) / ROT_SCALE
    return torch.cat([six, (ddf.double() / DEFOCUS_SCALE)[:, None]], dim=1).to(torch.float32)


def decode_outputs(out: torch.Tensor):
    """Network outputs -> (delta rotation (N,3,3) via Gram-Schmidt, defocus offset (N,) in A)."""
    o = out.double()
    eye = torch.eye(3, dtype=torch.float64, device=o.device)
    a1 = o[:, 0:3] * ROT_SCALE + eye[:, 0]
    a2 = o[:, 3:6] * ROT_SCALE + eye[:, 1]
    b1 = a1 / a1.norm(dim=1, keepdim=True)
    a2 = a2 - (b1 * a2).sum(dim=1, keepdim=True) * b1
    b2 = a2 / a2.norm(dim=1, keepdim=True)
    b3 = torch.cross(b1, b2, dim=1)
    return torch.stack([b1, b2, b3], dim=2), o[:, 6] * DEFOCUS_SCALE


def angular_error_deg(ra: torch.Tensor, rb: torch.Tensor) -> torch.Tensor:
    tr = (ra.double() @ rb.double().transpose(-1, -2)).diagonal(dim1=-2, dim2=-1).sum(-1)
    return torch.rad2deg(torch.acos(torch.clamp((tr - 1) / 2, -1.0, 1.0)))


@dataclass
class TrainReport:
    steps: int
    final_loss: float
    seconds: float
    samples: int


def train(net: ProposalNet, inputs: torch.Tensor, targets: torch.Tensor, epochs: int = 6, batch: int = 256,
          lr: float = 1e-3, seed: int = 0) -> TrainReport:
    """Minibatch Adam with cosine learning-rate decay, all through the CUDA kernels."""
    import time

    n = inputs.shape[0]
    g = torch.Generator().manual_seed(seed)
    steps_per_epoch = max(1, n // batch)
    total = epochs * steps_per_epoch
    t0 = time.perf_counter()
    loss = None
    k = 0
    for _ in range(epochs):
        perm = torch.randperm(n, generator=g).to(inputs.device)
        for sidx in range(steps_per_epoch):
            idx = perm[sidx * batch : (sidx + 1) * batch]
            out = net.forward(inputs[idx])
            loss, dout = net.loss_and_grad(out, targets[idx])
            net.backward(dout)
            cur = lr * 0.5 * (1 + math.cos(math.pi * k / total))
            net.adam_step(cur)
            k += 1
    torch.cuda.synchronize(net.dev)
    net.check_device_status()
    return TrainReport(k, float(loss.item()) if loss is not None else float("nan"), time.perf_counter() - t0,
                       k * batch)


def predict(net: ProposalNet, inputs: torch.Tensor, batch: int = 1024):
    outs = []
    for a in range(0, inputs.shape[0], batch):
        outs.append(net.forward(inputs[a : a + batch]))
    net.check_device_status()
    return torch.cat(outs)


# ---- refinement with proposals ------------------------------------------------------
def refine_with_proposals(net: ProposalNet | None, kwargs: dict, device, small_offsets: torch.Tensor,
                          small_defocus: torch.Tensor, batch_size: int = 32, margin: float = 0.0,
                          proposal: str = "network"):
    """Proposal -> plain local grid on a small neighbourhood of the proposal;
    the full plain grid is the fallback for every particle whose proposal
    search does not beat the score of its starting pose (all defocus offsets
    of the full grid at the starting orientation).

    ``proposal`` = "network" (the trained CNN) or "gauss_newton" (the
    linearised step of the network's own input channels, no network: the
    ablation that measures what the network adds).

    Returns (result dict like core_refine_template, info dict)."""
    from .backend.core_refine_template import _ctf_params, core_refine_template

    if proposal not in ("network", "gauss_newton"):
        raise ValueError(f"proposal must be 'network' or 'gauss_newton', got {proposal!r}")
    dev = torch.device(device)
    # the template and the per-particle images, filters and statistics maps go
    # to the device once: the input builder and the refinement calls below
    # would each upload them again
    kwargs = dict(kwargs)
    for k in ("particle_stack_dft", "template_dft", "corr_mean", "corr_std", "projective_filters"):
        if isinstance(kwargs.get(k), torch.Tensor):
            kwargs[k] = kwargs[k].to(dev)
    ctf = _ctf_params(kwargs["ctf_kwargs"])
    e0 = kwargs["euler_angles"].to(torch.float64)
    r0 = rot.euler_zyz_to_rotmat(e0)
    x, gn = make_inputs(kwargs["particle_stack_dft"], kwargs["template_dft"], r0.float(), kwargs["defocus_u"],
                        kwargs["defocus_v"], kwargs["defocus_angle"], ctf, dev)
    if proposal == "network":
        delta, ddf = decode_outputs(predict(net, x))
    else:
        delta, ddf = gauss_newton_proposal(gn)
    r_prop = delta.cpu() @ r0
    e_prop = rot.rotmat_to_euler_zyz(r_prop).to(torch.float32)
    prop = dict(kwargs)
    prop["euler_angle_offsets"] = small_offsets
    prop["defocus_offsets"] = small_defocus
    prop["euler_angles"] = e_prop
    prop["defocus_u"] = kwargs["defocus_u"] + ddf.cpu().float()
    prop["defocus_v"] = kwargs["defocus_v"] + ddf.cpu().float()
    res_p = core_refine_template(**prop, device=dev, batch_size=batch_size)
    start = dict(kwargs)
    start["euler_angle_offsets"] = torch.zeros((1, 3))
    res_s = core_refine_template(**start, device=dev, batch_size=batch_size)
    fb = res_p["refined_z_score"] <= res_s["refined_z_score"] + margin
    res = {k: v.clone() for k, v in res_p.items()}
    # offsets returned relative to the particle's own starting defocus, like the plain grid
    res["refined_defocus_offset"] = res_p["refined_defocus_offset"] + ddf.cpu().float()
    n_fb = int(fb.sum())
    if n_fb:
        sel = torch.nonzero(fb).flatten()
        sub = {k: (v[sel.to(v.device)] if isinstance(v, torch.Tensor) and v.shape[:1] == fb.shape else v)
               for k, v in kwargs.items()}
        res_f = core_refine_template(**sub, device=dev, batch_size=batch_size)
        for k in res:
            res[k][sel] = res_f[k].to(res[k].dtype)
    n = fb.numel()
    K_small = int(small_offsets.shape[0]) * int(small_defocus.shape[0])
    K_full = int(kwargs["euler_angle_offsets"].shape[0]) * int(kwargs["defocus_offsets"].shape[0])
    info = {"fallback": n_fb, "particles": n, "small_grid_correlations": K_small,
            "full_grid_correlations": K_full,
            "correlations_per_particle": K_small + int(kwargs["defocus_offsets"].shape[0])
            + K_full * n_fb / max(1, n)}
    return res, info


def load_weights(net: ProposalNet, path: str) -> None:
    with np.load(path) as z:
        net.load({k: z[k].astype(np.float32) for k in z.files if k != "layers"})


def stored_layers(path: str):
    """The layer list saved with the weights (files without one hold LAYERS)."""
    with np.load(path) as z:
        if "layers" not in z.files:
            return list(LAYERS)
        return [(k, int(a), int(b), int(s), bool(r)) for k, a, b, s, r in json.loads(str(z["layers"]))]


def load_net(path: str, device) -> ProposalNet:
    """A network built from the layer list stored with the weights, weights loaded."""
    net = ProposalNet(device, layers=stored_layers(path))
    load_weights(net, path)
    return net


def save_weights(net: ProposalNet, path: str) -> None:
    np.savez_compressed(path, layers=np.array(json.dumps([list(l) for l in net.layers])),
                        **{k: v.astype(np.float16) for k, v in net.state().items()})
