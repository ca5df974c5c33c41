"""Train the refinement proposal network on particles the method simulates.

    python -m leopard_em_gb300.train_proposal --n-train 500000 --out weights.npz

Data: ``synthetic.simulate_particles`` for the refinement configuration
(288^2 crops, 256^3 Gaussian-blob template, poses perturbed by up to 3
degrees, defocus offsets up to +-400 A, shifts up to +-3 px, SNR 0.05-0.2),
turned into network inputs by the CUDA input builder.  Training runs entirely
through the package's CUDA kernels (forward, backward, Adam).  Prints the
held-out rotation / defocus errors of the starting poses, of the Gauss-Newton
step alone and of the network.
"""

from __future__ import annotations

import argparse
import json
import time

import torch

from . import preprocess as pp
from . import proposal as pr
from . import synthetic as sy
from .backend.core_refine_template import _ctf_params


def build_dataset(cfg, n, seed, device, chunk=4096):
    vol, centres = sy.blob_volume(cfg.template_size, cfg.n_blobs, cfg.blob_sigma, cfg.blob_radius, cfg.seed,
                                  device=device)
    tdft = pp.volume_to_rfft_fourier_slice(vol).to(torch.complex64)
    del vol
    cp = _ctf_params(dict(voltage=300.0, spherical_aberration=2.7, amplitude_contrast_ratio=0.07, ctf_B_factor=0.0,
                          phase_shift=0.0, pixel_size=cfg.pixel_size))
    xs, ts, extra = [], [], []
    for a in range(0, n, chunk):
        m = min(chunk, n - a)
        sim = sy.simulate_particles(cfg, centres, m, seed + a, device=device)
        full = torch.full((m,), cfg.defocus)
        x, gn = pr.make_inputs(sim["particle_dft"], tdft, sim["r_start"].float(), full, full, torch.zeros(m), cp,
                               device)
        del sim["particle_dft"]
        xs.append(x)
        ts.append(pr.targets_from(sim["r_true"], sim["r_start"], sim["ddf"]))
        extra.append({"r_true": sim["r_true"], "r_start": sim["r_start"], "ddf": sim["ddf"], "gn": gn.cpu()})
    cat = {k: torch.cat([e[k] for e in extra]) for k in extra[0]}
    return torch.cat(xs), torch.cat(ts).to(device), cat


def evaluate(net, x, truth):
    delta, ddf = pr.decode_outputs(pr.predict(net, x))
    r_prop = delta.cpu() @ truth["r_start"]
    d_gn, ddf_gn = pr.gauss_newton_proposal(truth["gn"])
    r_gn = d_gn @ truth["r_start"]
    return {
        "rotation_error_deg": {"start": pr.angular_error_deg(truth["r_start"], truth["r_true"]).mean().item(),
                               "gauss_newton": pr.angular_error_deg(r_gn, truth["r_true"]).mean().item(),
                               "network": pr.angular_error_deg(r_prop, truth["r_true"]).mean().item()},
        "defocus_error_A": {"start": truth["ddf"].abs().mean().item(),
                            "gauss_newton": (ddf_gn - truth["ddf"]).abs().mean().item(),
                            "network": (ddf.cpu() - truth["ddf"]).abs().mean().item()},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=500000)
    ap.add_argument("--n-test", type=int, default=2048)
    ap.add_argument("--epochs", type=int, default=4)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", required=True)
    ap.add_argument("--layers", default=None,
                    help="JSON list of [kind, in, out, stride, relu] layers (default: proposal.LAYERS)")
    ap.add_argument("--compare-layers", default=None,
                    help="JSON layer list of a second network trained on the same data for comparison")
    ap.add_argument("--compare-out", default=None, help="where to save the second network's weights")
    args = ap.parse_args()
    dev = torch.device("cuda:0")
    cfg = sy.CONFIG_REFINE
    t0 = time.perf_counter()
    x, t, _ = build_dataset(cfg, args.n_train, 1000, dev)
    x_te, _, truth = build_dataset(cfg, args.n_test, 10 ** 8, dev)
    t_data = time.perf_counter() - t0
    runs = [(args.layers, args.out)]
    if args.compare_layers:
        runs.append((args.compare_layers, args.compare_out))
    for spec, out in runs:
        layers = json.loads(spec) if spec else None
        net = pr.ProposalNet(dev, seed=0, layers=layers)
        rep = pr.train(net, x, t, epochs=args.epochs, batch=args.batch, lr=args.lr)
        if out:
            pr.save_weights(net, out)
        ev = evaluate(net, x_te, truth)
        print(json.dumps({"n_train": args.n_train, "epochs": args.epochs, "layers": net.layers,
                          "params": net.n_params, "data_seconds": t_data, "train_seconds": rep.seconds,
                          "steps": rep.steps, "final_loss": rep.final_loss, "held_out": ev}), flush=True)


if __name__ == "__main__":
    main()
