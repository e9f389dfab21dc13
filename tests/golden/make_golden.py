"""Writes the golden fixtures under tests/golden/ from the CPU oracle.

The reference ships no stored outputs, so these vectors come from the oracle (which the
known-answer tests pin to the physics and to the reference's rules).  Each fixture
stores its inputs (plasma and beam arrays, grid) and the oracle's outputs for one 3D
step: per-slice iteration counts and final residuals, the e, b, psi and q_spe stores at
every slice, and the surviving plasma.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

CASES = {
    # name: (nr, nz, M, dr, dxi, ppc, ntheta, uth, beam (n_b, sigma_r, sigma_xi, center, num, x0), push_type)
    "loop_m2_nr48": (48, 24, 2, 0.05, 0.05, (2, 1), 8, 1e-3, (2.0, 0.4, 0.3, 0.45, 2000, 0.05), O.PUSH_ROBUST),
    "loop_m1_nr40_std": (40, 20, 1, 0.06, 0.05, (2, 1), 8, 0.0, (1.5, 0.5, 0.3, 0.4, 1500, 0.0), O.PUSH_STD),
}


def inputs(name):
    nr, nz, M, dr, dxi, ppc, nth, uth, bm, push = CASES[name]
    g = O.grid(nr, nz, M, dr, dxi)
    pl = O.load_plasma(g, 11, ppc[0], ppc[1], nth, uth=(uth, uth, uth))
    nb, sr, sz, c, num, x0 = bm
    Q = nb * (2 * np.pi) ** 1.5 * sr * sr * sz
    beam = O.load_beam(g, 12, num, Q, -1.0, 20000.0, (x0, 0.0, c), (sr, sr, sz), (x0 - 5 * sr, -5 * sr, 0.0),
                       (x0 + 5 * sr, 5 * sr, min(nz * dxi, c + 5 * sz)), uth=(2e-3, 2e-3, 0.0))
    return g, pl, beam, push


def run(name, g, pl, beam, push):
    sim = O.Sim(g, iter_max=30, iter_reltol=1e-6, dt3d=5.0, sp_push_type=push, sp_npmax=pl.n,
                beams=[(-1.0, O.PUSH3_REDUCED, beam.n)])
    sim.set_plasma(pl)
    sim.set_beam(0, beam)
    iters, rel = sim.run_3dstep()
    out = {"iters": iters, "rel": rel}
    for f in ("e", "b", "psi", "q_spe"):
        out["store_" + f] = sim.store(f)[:g.nz]
    p = sim.plasma()
    for k in O.Plasma.NAMES:
        out["out_" + k] = getattr(p, k)
    b = sim.beam(0)
    for k in O.Beam.NAMES:
        out["beam_out_" + k] = getattr(b, k)
    return out


def main():
    for name in CASES:
        g, pl, beam, push = inputs(name)
        out = run(name, g, pl, beam, push)
        arrays = {"grid": np.array([g.nr, g.nz, g.max_mode, g.dr, g.dxi, g.relax_fac, push], np.float64)}
        for k in O.Plasma.NAMES:
            arrays["in_" + k] = getattr(pl, k)
        for k in O.Beam.NAMES:
            arrays["beam_in_" + k] = getattr(beam, k)
        arrays.update(out)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **arrays)
        print(path, os.path.getsize(path), "bytes; mean iterations", float(np.mean(out["iters"])))


if __name__ == "__main__":
    main()
