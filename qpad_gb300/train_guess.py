"""Trains the learned predictor-corrector guess for c2-shaped runs and writes the weights.

    python -m qpad_gb300.train_guess [--runs 8] [--epochs 30] [--out qpad_gb300/weights/guess_c2.npz]

Training data come from the plain solver (mixed path) on c2-shaped decks (nr=512, M=2,
1024 slices) whose driver peak density is drawn from U[1, 10] (seed 3) with a witness of
twice that density; every slice j >= 3 of every mode is one sample.  Both nets are
trained with Adam by the library's own GPU kernels, then evaluated on a held-out driver
(n_b = 3): B-perp iterations per slice with and without the guess.
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
        sim = build_simulation(c2_variant(n_b, 100 + k), precision=K.PREC_MIXED)
        it, _ = sim.run_3d_step()
        (a0, b0), (a1, b1) = LR.dataset(sim)
        x0.append(a0); t0.append(b0); x1.append(a1); t1.append(b1)
        info.append({"n_b": n_b, "iters_per_slice": float(it.mean())})
        sim.close()
    return (np.concatenate(x0), np.concatenate(t0)), (np.concatenate(x1), np.concatenate(t1)), info


def evaluate(net0, net1, n_b: float = 3.0, apply_b=True, apply_j=True, weight=1.0):
    d = c2_variant(n_b, 999)
    a = build_simulation(d, precision=K.PREC_MIXED)
    ia, _ = a.run_3d_step()
    b = build_simulation(d, precision=K.PREC_MIXED)
    LR.attach(b, net0, net1)
    LR.configure(b, apply_b, apply_j, weight)
    ib, _ = b.run_3d_step()
    a.close()
    b.close()
    return float(ia.mean()), float(ib.mean())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--runs", type=int, default=8)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--out", default=DEFAULT_OUT)
    args = ap.parse_args()
    (x0, t0), (x1, t1), info = generate(args.runs)
    net0 = LR.ConvNet(*LR.CHANNELS[0], seed=1)
    net1 = LR.ConvNet(*LR.CHANNELS[1], seed=2)
    l0 = net0.train(x0, t0, epochs=args.epochs, batch=64, lr=1e-3, seed=1)
    l1 = net1.train(x1, t1, epochs=args.epochs, batch=64, lr=1e-3, seed=2)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    LR.save(args.out, net0, net1)
    plain, guessed = evaluate(net0, net1)
    print(json.dumps({"runs": info, "samples": [len(x0), len(x1)],
                      "final_loss_rel": [float(l0[-1] / np.mean(t0 ** 2)), float(l1[-1] / np.mean(t1 ** 2))],
                      "held_out_iters_per_slice": {"plain": plain, "guess": guessed}}))


if __name__ == "__main__":
    main()
