"""Proposal network: CUDA kernels against the CPU oracle (forward, gradients of
every layer, Adam, input builder) and the gain of a network trained on the
method's simulated particles over the starting poses."""

import math

import numpy as np
import pytest
import torch

from leopard_em_gb300 import proposal as pr
from leopard_em_gb300 import synthetic as sy
from leopard_em_gb300.backend.core_refine_template import _ctf_params
from oracle import ref_cnn

pytestmark = pytest.mark.gpu
DEV = torch.device("cuda:0")


def _rel(a, b):
    a, b = a.double().cpu(), b.double().cpu()
    return float((a - b).norm() / b.norm().clamp_min(1e-30))


def test_forward_and_gradients_match_oracle():
    net = pr.ProposalNet(DEV, seed=3)
    g = torch.Generator().manual_seed(0)
    for b in net.b:  # non-zero biases exercise the bias paths
        b.copy_(0.05 * torch.randn(b.shape, generator=g).to(DEV))
    x = torch.randn(5, pr.CHANNELS, 64, 64, generator=g).to(torch.bfloat16)
    tgt = torch.randn(5, 7, generator=g)
    out = net.forward(x.to(DEV))
    loss, dout = net.loss_and_grad(out, tgt.to(DEV))
    net.backward(dout)
    torch.cuda.synchronize()
    r_out, r_loss, r_gw, r_gb = ref_cnn.loss_and_grads(x.double(), [w.cpu() for w in net.w],
                                                       [b.cpu() for b in net.b], tgt, pr.LAYERS)
    assert _rel(out, r_out) < 1e-2
    assert abs(float(loss) - float(r_loss)) <= 1e-2 * float(r_loss)
    for i in range(len(pr.LAYERS)):
        assert _rel(net.gw[i], r_gw[i]) < 2e-2, f"weight grad layer {i}: {_rel(net.gw[i], r_gw[i])}"
        assert _rel(net.gb[i], r_gb[i]) < 2e-2, f"bias grad layer {i}"


def test_adam_step_matches_formula():
    net = pr.ProposalNet(DEV, seed=1)
    w0 = net.w[2].clone()
    net.gw[2].copy_(torch.randn_like(w0))
    g = net.gw[2].clone()
    for gg in net.gb:
        gg.zero_()
    net.adam_step(1e-2)
    torch.cuda.synchronize()
    m = 0.1 * g
    v = 0.001 * g * g
    expect = w0 - 1e-2 * (m / 0.1) / (torch.sqrt(v / 0.001) + 1e-8)
    assert torch.allclose(net.w[2], expect, rtol=1e-5, atol=1e-6)
    assert torch.equal(net.wbf[2], net.w[2].to(torch.bfloat16))


def test_input_builder_matches_oracle():
    cfg = sy.RefineConfig(crop=128, template_size=64, n_blobs=100, blob_radius=20.0)
    kw, truth = sy.make_refine_workload(cfg, 3)
    R = truth["r_start"].float()
    ctf = kw["ctf_kwargs"]
    x, gn = pr.make_inputs(kw["particle_stack_dft"], kw["template_dft"], R, kw["defocus_u"], kw["defocus_v"],
                           kw["defocus_angle"], _ctf_params(ctf), DEV)
    got = x.cpu().double()
    ref = ref_cnn.make_inputs(kw["particle_stack_dft"], kw["template_dft"], R, kw["defocus_u"], kw["defocus_v"],
                              kw["defocus_angle"], ctf)
    assert got.shape == (3, pr.CHANNELS, 64, 64)
    for ch in range(pr.IMAGE_CHANNELS):
        assert _rel(got[:, ch], ref[:, ch]) < 2e-2, f"channel {ch}: {_rel(got[:, ch], ref[:, ch])}"
    # Gauss-Newton step from the GPU's own bf16 channels
    ref_gn = ref_cnn.gauss_newton(got[:, : pr.IMAGE_CHANNELS])
    assert _rel(gn.cpu()[:, :6], ref_gn[:, :6]) < 1e-3
    scale = torch.tensor([0.5, 0.5, 1 / 3, 1 / 3, 1 / 3, 0.25], dtype=torch.float64)
    for a in range(6):
        assert torch.allclose(got[:, 6 + a, 7, 9], (gn.cpu()[:, a].double() * scale[a]), rtol=1e-2, atol=1e-3)


def test_trained_network_improves_on_starting_poses():
    """Train on 6144 simulated particles; on 256 held-out ones the proposals must
    cut the rotation and defocus errors of the starting poses."""
    cfg = sy.RefineConfig(crop=128, template_size=64, n_blobs=120, blob_radius=22.0, snr_range=(0.3, 0.6))
    vol, centres = sy.blob_volume(64, 120, cfg.blob_sigma, 22.0, cfg.seed)
    from leopard_em_gb300 import preprocess as pp

    tdft = pp.volume_to_rfft_fourier_slice(vol).to(torch.complex64)
    ctf = dict(voltage=300.0, spherical_aberration=2.7, amplitude_contrast_ratio=0.07, ctf_B_factor=0.0,
               phase_shift=0.0, pixel_size=cfg.pixel_size)
    cp = _ctf_params(ctf)

    def batch(n, seed):
        sim = sy.simulate_particles(cfg, centres, n, seed, device=DEV)
        full = torch.full((n,), cfg.defocus)
        x, gn = pr.make_inputs(sim["particle_dft"], tdft, sim["r_start"].float(), full, full, torch.zeros(n), cp, DEV)
        sim["gn"] = gn
        return x, sim

    xs, ts = [], []
    for k in range(3):
        x, sim = batch(2048, 100 + k)
        xs.append(x)
        ts.append(pr.targets_from(sim["r_true"], sim["r_start"], sim["ddf"]))
    x_tr, t_tr = torch.cat(xs), torch.cat(ts).to(DEV)
    net = pr.ProposalNet(DEV, seed=0)
    rep = pr.train(net, x_tr, t_tr, epochs=10, batch=256, lr=2e-3)
    assert math.isfinite(rep.final_loss)
    x_te, sim = batch(256, 999)
    delta, ddf = pr.decode_outputs(pr.predict(net, x_te))
    r_prop = delta.cpu() @ sim["r_start"]
    err_start = pr.angular_error_deg(sim["r_start"], sim["r_true"]).mean().item()
    err_prop = pr.angular_error_deg(r_prop, sim["r_true"]).mean().item()
    dferr_start = sim["ddf"].abs().mean().item()
    dferr_prop = (ddf.cpu() - sim["ddf"]).abs().mean().item()
    d_gn, ddf_gn = pr.gauss_newton_proposal(sim["gn"])
    err_gn = pr.angular_error_deg(d_gn @ sim["r_start"], sim["r_true"]).mean().item()
    print(f"rotation error start {err_start:.3f} gauss-newton {err_gn:.3f} network {err_prop:.3f} deg; "
          f"defocus error {dferr_start:.1f} -> {dferr_prop:.1f} A")
    assert err_prop < 0.8 * err_start
    assert dferr_prop < 0.8 * dferr_start


def _layer_ws(L, fn, *args):
    import ctypes

    n = ctypes.c_size_t(0)
    assert fn(*args, ctypes.byref(n)) == 0
    return torch.empty(n.value, dtype=torch.uint8, device=DEV)


@pytest.mark.parametrize("N,Cin,H,Cout,stride", [(3, 5, 13, 7, 1), (2, 12, 17, 33, 2), (1, 128, 6, 128, 1),
                                                 (5, 3, 31, 64, 2)])
def test_conv_layer_odd_shapes_match_torch(N, Cin, H, Cout, stride):
    """Tensor-core conv3x3 (forward, input, weight and bias gradients) on shapes
    that fill no tile evenly, against torch's FP32 convolution of the same
    BF16-rounded operands.  Tolerance 1e-2 relative: the output gradient enters
    the MMA rounded to BF16."""
    import ctypes

    from leopard_em_gb300._native import lib

    L = lib()
    g = torch.Generator().manual_seed(N * 100 + Cin)
    x = torch.randn(N, Cin, H, H, generator=g).to(torch.bfloat16)
    w = (0.2 * torch.randn(Cout, Cin, 3, 3, generator=g)).to(torch.bfloat16)
    b = torch.randn(Cout, generator=g)
    Ho = (H - 1) // stride + 1
    gy = torch.randn(N, Cout, Ho, Ho, generator=g)
    xd, wd, bd, gd = x.to(DEV), w.to(DEV), b.to(DEV), gy.to(DEV)
    ws = _layer_ws(L, L.lgb_nn_conv3x3_workspace_size, N, Cin, H, H, Cout, stride)
    st = torch.zeros(1, dtype=torch.int32, device=DEV)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    y = torch.empty(N, Cout, Ho, Ho, dtype=torch.bfloat16, device=DEV)
    assert L.lgb_nn_conv3x3_forward(N, Cin, H, H, Cout, stride, 0, xd.data_ptr(), wd.data_ptr(), bd.data_ptr(),
                                    y.data_ptr(), ws.data_ptr(), ws.numel(), st.data_ptr(), s) == 0
    dx = torch.empty(N, Cin, H, H, device=DEV)
    dw = torch.empty(Cout, Cin, 3, 3, device=DEV)
    db = torch.empty(Cout, device=DEV)
    assert L.lgb_nn_conv3x3_backward(N, Cin, H, H, Cout, stride, xd.data_ptr(), wd.data_ptr(), gd.data_ptr(),
                                     dx.data_ptr(), dw.data_ptr(), db.data_ptr(), ws.data_ptr(), ws.numel(),
                                     st.data_ptr(), s) == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    xr = x.float().requires_grad_(True)
    wr = w.float().requires_grad_(True)
    br = b.clone().requires_grad_(True)
    yr = torch.nn.functional.conv2d(xr, wr, br, stride=stride, padding=1)
    yr.backward(gy.to(torch.bfloat16).float())
    assert _rel(y.float(), yr.detach()) < 1e-2
    assert _rel(dx, xr.grad) < 1e-2
    assert _rel(dw, wr.grad) < 1e-2
    assert _rel(db, br.grad) < 1e-2


@pytest.mark.parametrize("N,In,Out", [(1, 5, 7), (37, 200, 130), (300, 2048, 1152), (129, 64, 600)])
def test_linear_layer_odd_shapes_match_torch(N, In, Out):
    """Tensor-core linear layer (forward with ReLU into BF16 and FP32 outputs,
    input, weight and bias gradients) against torch FP32 on the same
    BF16-rounded operands."""
    import ctypes

    from leopard_em_gb300._native import lib

    L = lib()
    g = torch.Generator().manual_seed(N + In + Out)
    x = torch.randn(N, In, generator=g).to(torch.bfloat16)
    w = (torch.randn(Out, In, generator=g) / math.sqrt(In)).to(torch.bfloat16)
    b = torch.randn(Out, generator=g)
    gy = torch.randn(N, Out, generator=g)
    xd, wd, bd, gd = x.to(DEV), w.to(DEV), b.to(DEV), gy.to(DEV)
    ws = _layer_ws(L, L.lgb_nn_linear_workspace_size, N, In, Out)
    st = torch.zeros(1, dtype=torch.int32, device=DEV)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ybf = torch.empty(N, Out, dtype=torch.bfloat16, device=DEV)
    yf = torch.empty(N, Out, device=DEV)
    assert L.lgb_nn_linear_forward(N, In, Out, 1, xd.data_ptr(), wd.data_ptr(), bd.data_ptr(), ybf.data_ptr(),
                                   yf.data_ptr(), ws.data_ptr(), ws.numel(), st.data_ptr(), s) == 0
    dx = torch.empty(N, In, device=DEV)
    dw = torch.empty(Out, In, device=DEV)
    db = torch.empty(Out, device=DEV)
    assert L.lgb_nn_linear_backward(N, In, Out, xd.data_ptr(), wd.data_ptr(), gd.data_ptr(), dx.data_ptr(),
                                    dw.data_ptr(), db.data_ptr(), ws.data_ptr(), ws.numel(), st.data_ptr(), s) == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = torch.relu(x.float() @ w.float().t() + b)
    assert _rel(yf, ref) < 1e-4
    assert torch.equal(ybf.cpu(), yf.cpu().to(torch.bfloat16))
    gq = gy.to(torch.bfloat16).float()
    assert _rel(dx, gq @ w.float()) < 1e-2
    assert _rel(dw, gq.t() @ x.float()) < 1e-2
    assert _rel(db, gq.sum(0)) < 1e-2
