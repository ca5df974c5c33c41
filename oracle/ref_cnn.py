"""CPU oracle of the refinement proposal network (TEST INFRASTRUCTURE ONLY).

Restates, in float64 torch with autograd, the network that
``leopard_em_gb300/csrc/nn.cu`` computes: 3x3 convolutions (pad 1, stride 1 or
2) and linear layers with ReLU, weights rounded to bfloat16, every stored
activation rounded to bfloat16 (straight-through: the rounding passes the
gradient unchanged, as the CUDA backward does), mean-squared-error loss.
Also restates the input builder ``lgb_nn_make_inputs``: the low-frequency
band of a particle spectrum and the template's central slice at a rotation
on the same physical frequencies times the CTF, inverse transformed and
standardised.  There is no reference counterpart (Leopard-EM has no learned
component); the slice follows the same restatement as ref_match_template.
"""

from __future__ import annotations

import math

import torch
import torch.nn.functional as F

from . import ref_match_template as mt
from . import ref_refine_template as rr


def bf16(x: torch.Tensor) -> torch.Tensor:
    return x.to(torch.bfloat16).to(torch.float64)


def _st_round(x):
    return x + (bf16(x) - x).detach()


def forward(x, weights, biases, layers):
    """x: (N, 2, 64, 64) float64 (bf16 values). Returns float64 (N, 7)."""
    a = x
    for i, (kind, cin, cout, stride, relu) in enumerate(layers):
        w = bf16(weights[i])
        if kind == "conv":
            a = F.conv2d(a, w, biases[i], stride=stride, padding=1)
        else:
            a = a.reshape(a.shape[0], -1) @ w.T + biases[i]
        if relu:
            a = torch.relu(a)
        if i < len(layers) - 1:
            a = _st_round(a)
    return a


def loss_and_grads(x, weights, biases, target, layers):
    ws = [w.detach().clone().double().requires_grad_(True) for w in weights]
    bs = [b.detach().clone().double().requires_grad_(True) for b in biases]
    out = forward(x.double(), ws, bs, layers)
    loss = ((out - target.double()) ** 2).sum(dim=1).mean()
    loss.backward()
    return out.detach(), loss.detach(), [w.grad for w in ws], [b.grad for b in bs]


def _slice_band(template_dft, R, fy, fx):
    d = template_dft.shape[0]
    zyx = torch.stack([torch.zeros_like(fy), fy, fx], dim=-1)
    r = zyx @ torch.flip(R, dims=(0, 1)).T
    conj = r[..., 2] < 0
    r = torch.where(conj[..., None], -r, r)
    coords = r * d + torch.tensor([d // 2, d // 2, 0], dtype=torch.float64)
    smp = mt._trilinear_zero_outside(template_dft.to(torch.complex128), coords)
    smp = -torch.where(conj, smp.conj(), smp)  # contrast-flipped, as the search's slices
    smp[0, 0] = 0
    return smp


def make_inputs(particle_dft, template_dft, rotations, defocus_u, defocus_v, defocus_angle, ctf, band=64):
    """(P, 6, band, band) float64: particle band re-centred from the crop centre
    to the frame origin and shift-aligned to the reference
    (peak of the band cross-correlation, parabolic sub-pixel, |shift| <= band/4)
    and standardised; reference (slice at R0 x CTF) standardised; 1-degree
    rotation finite differences about the image x, y, z axes and the defocus
    derivative (per 100 A) of the reference, mean-subtracted and divided by the
    reference's std."""
    P, H, wc = particle_dft.shape
    W = 2 * (wc - 1)
    G, GH = band, band // 2
    rows = torch.cat([torch.arange(GH), torch.arange(H - GH, H)])
    ky = torch.cat([torch.arange(GH), torch.arange(-GH, 0)]).double()
    kx = torch.arange(GH + 1).double()
    fy = (ky / H)[:, None].expand(G, GH + 1)
    fx = (kx / W)[None, :].expand(G, GH + 1)
    kyA = (ky / H / ctf["pixel_size"])[:, None].expand(G, GH + 1)
    kxA = (kx / W / ctf["pixel_size"])[None, :].expand(G, GH + 1)
    k2 = kxA**2 + kyA**2
    ang = torch.atan2(kyA, kxA)
    lam = rr.electron_wavelength_angstrom(ctf["voltage"])
    amp = ctf["amplitude_contrast_ratio"]
    dl = math.radians(1.0)
    c, sn = math.cos(dl), math.sin(dl)
    Ds = [torch.tensor(m, dtype=torch.float64) for m in (
        [[1, 0, 0], [0, c, -sn], [0, sn, c]], [[c, 0, sn], [0, 1, 0], [-sn, 0, c]], [[c, -sn, 0], [sn, c, 0], [0, 0, 1]])]

    def irfft(spec):
        return torch.fft.irfft2(spec, s=(G, G)) * (G * G)

    outs = []
    for p in range(P):
        R0 = rotations[p].reshape(3, 3).to(torch.float64)
        dfm = 0.5 * (float(defocus_u[p]) + float(defocus_v[p]))
        ast = 0.5 * abs(float(defocus_u[p]) - float(defocus_v[p]))
        dfe = dfm + ast * torch.cos(2 * (ang - math.radians(float(defocus_angle[p]))))
        chi = (-math.pi * lam * k2 * dfe + 0.5 * math.pi * ctf["spherical_aberration"] * 1e7 * lam**3 * k2**2
               - math.radians(ctf["phase_shift"]) - math.atan(amp / math.sqrt(1 - amp**2)))
        env = torch.exp(-ctf["ctf_B_factor"] * k2 / 4)
        ctfv = -torch.sin(chi) * env
        dctf = -torch.cos(chi) * (-math.pi * lam * k2) * 100.0 * env
        pspec = particle_dft[p][rows][:, : GH + 1].to(torch.complex128).clone()
        # particles sit at the crop centre; re-centre on the frame origin
        pspec = pspec * (1 - 2 * ((ky[:, None].long() + kx[None, :].long()) % 2))
        pspec[0, 0] = 0
        r0 = _slice_band(template_dft, R0, fy, fx)
        cc = irfft(pspec * torch.conj(r0 * ctfv))
        sy = torch.cat([torch.arange(GH), torch.arange(-GH, 0)])
        ok = (sy.abs() <= G // 4)[:, None] & (sy.abs() <= G // 4)[None, :]
        e = int(torch.argmax(torch.where(ok, cc, torch.full_like(cc, -float("inf")))))
        y, x = e // G, e % G
        c0 = cc[y, x]
        ym, yp, xm, xp = cc[(y - 1) % G, x], cc[(y + 1) % G, x], cc[y, (x - 1) % G], cc[y, (x + 1) % G]
        deny, denx = ym - 2 * c0 + yp, xm - 2 * c0 + xp
        dy = float(torch.clamp(0.5 * (ym - yp) / deny, -0.5, 0.5)) if deny < 0 else 0.0
        dx = float(torch.clamp(0.5 * (xm - xp) / denx, -0.5, 0.5)) if denx < 0 else 0.0
        shy = float(sy[y]) + dy
        shx = float(sy[x]) + dx
        ramp = torch.exp(2j * math.pi * (ky[:, None] * shy + kx[None, :] * shx) / G)
        img_p = irfft(pspec * ramp)
        ch = [(img_p - img_p.mean()) / img_p.std(unbiased=False)]
        img_r = irfft(r0 * ctfv)
        rs = img_r.std(unbiased=False)
        ch.append((img_r - img_r.mean()) / rs)
        for D in Ds:
            ra = _slice_band(template_dft, D @ R0, fy, fx)
            im = irfft((ra - r0) * ctfv)
            ch.append((im - im.mean()) / rs)
        im = irfft(r0 * dctf)
        ch.append((im - im.mean()) / rs)
        outs.append(torch.stack(ch))
    return torch.stack(outs)


def gauss_newton(x):
    """Restates lgb_nn_gauss_newton on input channels 0-5 (float64): J = [central
    differences of the reference along x and y (periodic), channels 2-5];
    a = <P,R>/<R,R>; delta = (J^T J + 1e-6 diag)^-1 J^T (P - a R) / a.
    Returns (P, 8): delta (6), a, residual fraction."""
    x = x.double()
    n = x.shape[0]
    P, R = x[:, 0], x[:, 1]
    gx = 0.5 * (torch.roll(R, -1, 2) - torch.roll(R, 1, 2))
    gy = 0.5 * (torch.roll(R, -1, 1) - torch.roll(R, 1, 1))
    J = torch.cat([gx[:, None], gy[:, None], x[:, 2:6]], 1).reshape(n, 6, -1)
    Pf, Rf = P.reshape(n, -1), R.reshape(n, -1)
    pr, rr, pp = (Pf * Rf).sum(1), (Rf * Rf).sum(1), (Pf * Pf).sum(1)
    a = pr / rr
    A = J @ J.transpose(1, 2)
    A = A + 1e-6 * torch.diag_embed(A.diagonal(dim1=1, dim2=2) + 1e-12)
    b = (J @ (Pf - a[:, None] * Rf)[:, :, None])[:, :, 0]
    delta = torch.linalg.solve(A, b) / a[:, None]
    res = (pp - 2 * a * pr + a * a * rr) / pp
    return torch.cat([delta, a[:, None], res[:, None]], 1)
