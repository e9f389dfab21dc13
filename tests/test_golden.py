"""Committed golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py).

CPU: the oracle, re-run on the stored inputs, still reproduces the stored outputs.
GPU: the CUDA path, run through the C ABI on the stored inputs, matches them within the
FP64 parity tolerance, with identical per-slice iteration counts and particle counts.
"""
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import sorted_rows, store_errors

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = sorted(glob.glob(os.path.join(HERE, "*.npz")))


def _load(path):
    z = np.load(path)
    nr, nz, M, dr, dxi, rf, push = z["grid"]
    g = O.grid(int(nr), int(nz), int(M), float(dr), float(dxi), relax_fac=float(rf))
    pl = O.Plasma(len(z["in_q"]))
    for k in O.Plasma.NAMES:
        getattr(pl, k)[:] = z["in_" + k]
    bm = O.Beam(len(z["beam_in_q"]))
    for k in O.Beam.NAMES:
        getattr(bm, k)[:] = z["beam_in_" + k]
    return z, g, pl, bm, int(push)


def test_fixtures_present():
    assert len(FIXTURES) >= 2


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_reproduces_golden(path):
    z, g, pl, bm, push = _load(path)
    sim = O.Sim(g, iter_max=30, iter_reltol=1e-6, dt3d=5.0, sp_push_type=push, sp_npmax=pl.n,
                beams=[(-1.0, O.PUSH3_REDUCED, bm.n)])
    sim.set_plasma(pl)
    sim.set_beam(0, bm)
    iters, rel = sim.run_3dstep()
    assert np.array_equal(iters, z["iters"])
    for f in ("e", "b", "psi", "q_spe"):
        np.testing.assert_allclose(sim.store(f)[:g.nz], z["store_" + f], rtol=1e-11, atol=1e-13)
    assert sim.plasma().n == len(z["out_q"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_gpu_matches_golden(path):
    import qpad_gb300 as Q
    z, g, pl, bm, push = _load(path)
    sim = Q.Simulation(g.nr, g.nz, g.max_mode, g.dr, g.dxi, relax_fac=g.relax_fac, iter_max=30, iter_reltol=1e-6,
                       dt=5.0)
    x = np.stack([pl.x, pl.y], 1)
    p = np.stack([pl.px, pl.py, pl.pz], 1)
    sim.add_species(x, p, pl.gamma, pl.psi, pl.q, push_type=push)
    sim.add_beam(np.stack([bm.x, bm.y, bm.z], 1), np.stack([bm.px, bm.py, bm.pz], 1), bm.q)
    iters, rel = sim.run_3d_step()
    assert np.array_equal(iters, z["iters"]), (iters, z["iters"])
    for f in ("e", "b", "psi", "q_spe"):
        got = np.stack([sim.fields[f].store(s) for s in range(1, g.nz + 1)])
        err = store_errors(got, z["store_" + f]).max()
        assert err < 1e-9, (f, err)
    x2, p2, g2, ps2, q2 = sim.species[0].download()
    assert len(q2) == len(z["out_q"])
    a = sorted_rows(q2, x2[:, 0], x2[:, 1])
    b = sorted_rows(z["out_q"], z["out_x"], z["out_y"])
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-11)
    bx, bp, bq = sim.beams[0].download()
    assert len(bq) == len(z["beam_out_q"])
    sim.close()
