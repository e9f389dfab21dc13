"""Trains the learned predictor-corrector guess and writes the weights.

    python -m qpad_gb300.train_guess [--runs 24] [--epochs 30] [--b-only] [--out qpad_gb300/weights/guess_c2.npz]

The committed weights/guess_c2.npz is the output of `--b-only` (24 runs, 30 epochs).  On the
held-out driver the m = 0 net predicts 84% of the variance of what the linear extrapolation
misses (relative MSE 0.16; the m >= 1 net 0.96), yet the loop with the nets takes more B-perp
iterations per slice (16.5) than the extrapolation alone (13.2) and than the carried guess
(15.4): the predicted residual moves the guess along directions the corrector then has to
undo.  The simulations default to the extrapolation; the nets stay an opt-in experiment.

The nets predict what the linear extrapolation of B-perp from the two previous slices misses
(qpad_guess_sample in include/qpad_gpu.h fixes the channels and their normalisation), so a
net that predicts nothing leaves the linear extrapolation.  Training data come from the plain
solver (mixed path) on c2-shaped decks (nr = 512, M = 2, 1024 slices) whose driver peak
density is drawn from U[1, 10] (seed 3), with a witness of twice that density.  Every slice j >= 3 of every mode is one
sample.  Both nets are trained with Adam by the library's own GPU kernels, then evaluated on a
held-out c2-shaped driver (n_b = 3): B-perp iterations per slice with the carried guess (the
reference), the linear extrapolation alone, and the extrapolation with the nets.
"""
from __future__ import annotations

import argparse
import json
import os

import numpy as np

from . import _capi as K
from . import decks
from . import learned as LR
from .runner import build_simulation

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "weights", "guess_c2.npz")


def c2_variant(n_b: float, seed: int, nz: int = 1024) -> decks.Deck:
    d = decks.c2()
    d.nz = nz
    d.seed = seed
    d.beams = [decks.BeamSpec(n_b, 0.3, 0.8, 2.4, 1_000_000, x0=0.03),
               decks.BeamSpec(2 * n_b, 0.2, 0.3, 6.4, 500_000)]
    return d


def generate(runs: int, seed: int = 3):
    rng = np.random.default_rng(seed)
    x0, t0, x1, t1, info = [], [], [], [], []
    for k in range(runs):
        n_b = float(rng.uniform(1.0, 10.0))
        d = c2_variant(n_b, 100 + k)
        sim = build_simulation(d, precision=K.PREC_MIXED)
        it, _ = sim.run_3d_step()
        (a0, b0), (a1, b1) = LR.dataset(sim)
        x0.append(a0); t0.append(b0); x1.append(a1); t1.append(b1)
        info.append({"deck": d.name, "n_b": n_b, "iters_per_slice": float(it.mean())})
        sim.close()
    return (np.concatenate(x0), np.concatenate(t0)), (np.concatenate(x1), np.concatenate(t1)), info


def evaluate(net0, net1, n_b: float = 3.0, weight=1.0, nz: int = 1024):
    """Iterations per slice on a held-out c2-shaped driver: carried guess, linear
    extrapolation, extrapolation + nets (with `weight` of the nets' correction)."""
    d = c2_variant(n_b, 999, nz=nz)
    out = {}
    for name, order, nets in (("carried", 0, False), ("extrapolated", 1, False), ("learned", 1, True)):
        s = build_simulation(d, precision=K.PREC_MIXED)
        s.set_guess_extrapolation(order)
        if nets:
            LR.attach(s, net0, net1)
            LR.configure(s, True, False, weight)
        it, _ = s.run_3d_step()
        out[name] = float(it.mean())
        s.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=24)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--b-only", action="store_true", help="train on the B-perp residual alone (J targets zeroed)")
    args = ap.parse_args()
    (x0, t0), (x1, t1), info = generate(args.runs)
    if args.b_only:
        t0[:, 2:] = 0.0
        t1[:, 4:] = 0.0
    rng = np.random.default_rng(4)
    nets, fits, losses = [], [], []
    for (x, t), ch, seed, nb in (((x0, t0), LR.CHANNELS[0], 1, 2), ((x1, t1), LR.CHANNELS[1], 2, 4)):
        idx = rng.permutation(len(x))
        nval = max(1, len(x) // 10)
        va, tr = idx[:nval], idx[nval:]
        net = LR.ConvNet(*ch, seed=seed)
        loss = net.train(x[tr], t[tr], epochs=args.epochs, batch=64, lr=1e-3, seed=seed)
        # held-out samples: the B-perp residual channels' mean squared error against their
        # mean square (1 = the net predicts nothing of what the extrapolation misses)
        y = net.predict(x[va])
        fits.append(float(np.mean((y[:, :nb] - t[va, :nb]) ** 2) / np.mean(t[va, :nb] ** 2)))
        losses.append(float(loss[-1] / np.mean(t[tr] ** 2)))
        nets.append(net)
    net0, net1 = nets
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    LR.save(args.out, net0, net1)
    print(json.dumps({"runs": info, "samples": [len(x0), len(x1)], "final_loss_rel": losses,
                      "held_out_b_residual_mse_rel": fits,
                      "held_out_iters_per_slice": evaluate(net0, net1)}))


if __name__ == "__main__":
    main()
