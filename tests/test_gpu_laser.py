"""GPU parity of the laser envelope and the PGC plasma species against the CPU oracle.

* Vacuum: the envelope advanced by 3D steps with no plasma (the penta-diagonal reduction
  alone) equals the oracle's to round-off.
* Plasma: a Gaussian pulse drives a wake in a cold uniform plasma of PGC species (robust and
  standard pushers; M = 1 and 2).  Over two 3D steps (the second sees the advanced envelope):
  identical per-slice iteration counts, every 3D store and the susceptibility store within
  1e-9, the advanced envelope within 1e-9, the plasma particles as a multiset.
* Refusals: the mixed path, nr not a power of two.
"""
import numpy as np
import pytest

import qpad_gb300 as Q
from oracle import oracle as O
from qpad_gb300 import _capi as K
from qpad_gb300 import lasers as LZ
from tests.helpers import plasma_to_oracle, sorted_rows, store_errors

pytestmark = pytest.mark.gpu

K0, A0, W0 = 10.0, 0.5, 1.0


def _deck(M, nr=64):
    return Q.decks.Deck("laser", nr=nr, nz=40, max_mode=M, dr=0.05, dxi=0.1, ppc=(2, 1), num_theta=8, uth=0.0,
                        seed=9, beams=[], iter_max=30, iter_reltol=1e-6, dt=2.0)


def _envelope(deck):
    return LZ.launch(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi, k0=K0, a0=A0, w0=W0, focal_distance=0.0,
                     lon=("sin2", 1.0, 0.0, 1.0), lon_center=1.5)


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_envelope_advance_in_vacuum_matches_oracle():
    deck = _deck(2)
    ar, ai = _envelope(deck)
    # a mode-2 part too, so that every mode's reduction runs
    ar[:, 3] = 0.3 * ar[:, 0]
    ai[:, 4] = -0.2 * ar[:, 0]
    g = O.grid(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi)
    osim = O.Sim(g, iter_max=5, dt3d=deck.dt, sp_npmax=1, lasers=[dict(k0=K0, iter=2, ar=ar, ai=ai)])
    osim.set_plasma(O.Plasma(0))
    sim = Q.Simulation(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi, iter_max=5, dt=deck.dt)
    lz = sim.add_laser(ar, ai, k0=K0, iteration=2)
    for _ in range(3):
        osim.run_3dstep(push_beams=False)
        sim.run_3d_step(push_beams=False)
    olr, oli = osim.laser(0)
    glr, gli = lz.download()
    assert _rel(glr, olr) < 1e-12 and _rel(gli, oli) < 1e-12
    assert np.abs(olr).max() > 0.1 * A0
    sim.close()


@pytest.mark.parametrize("M,push_type", [(1, O.PUSH_ROBUST_PGC), (2, O.PUSH_ROBUST_PGC), (1, O.PUSH_STD_PGC)])
def test_laser_wake_matches_oracle(M, push_type):
    deck = _deck(M)
    pl, _ = Q.deck_inputs(deck)
    ar, ai = _envelope(deck)
    g = O.grid(deck.nr, deck.nz, M, deck.dr, deck.dxi)
    osim = O.Sim(g, iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, dt3d=deck.dt, sp_push_type=push_type,
                 sp_npmax=len(pl[4]), lasers=[dict(k0=K0, iter=1, ar=ar, ai=ai)], sp_ppc_r=deck.ppc[0])
    sim = Q.Simulation(deck.nr, deck.nz, M, deck.dr, deck.dxi, iter_max=deck.iter_max,
                       iter_reltol=deck.iter_reltol, dt=deck.dt)
    sim.add_species(*pl, push_type=push_type, ppc_r=deck.ppc[0])
    lz = sim.add_laser(ar, ai, k0=K0, iteration=1)
    for step in range(2):
        osim.set_plasma(plasma_to_oracle(*pl))
        oit, _ = osim.run_3dstep(push_beams=False)
        if step:
            sim.species[0].reset()
        it, _ = sim.run_3d_step(push_beams=False)
        assert np.array_equal(it, oit), (step, it, oit)
        worst = {}
        for name in ("e", "b", "psi", "cu", "q_spe", "b_spe"):
            ref = osim.store(name)[:deck.nz]
            got = np.stack([sim.fields[name].store(s) for s in range(1, deck.nz + 1)])
            worst[name] = store_errors(got, ref).max()
        assert max(worst.values()) < 1e-9, (step, worst)
        ochi = osim.store("chi")[:deck.nz, :, 0]
        assert _rel(sim.chi_store(), ochi) < 1e-9
        olr, oli = osim.laser(0)
        glr, gli = lz.download()
        assert _rel(glr, olr) < 1e-9 and _rel(gli, oli) < 1e-9
    assert np.abs(osim.store("e")[:deck.nz, 0, 2, 1]).max() > 1e-3      # a wake
    opl = osim.plasma()
    x, p, gm, ps, q = sim.species[0].download()
    assert len(q) == opl.n
    np.testing.assert_allclose(sorted_rows(q, x[:, 0], x[:, 1]), sorted_rows(opl.q, opl.x, opl.y), rtol=1e-9,
                               atol=1e-11)
    sim.close()


def test_laser_refusals():
    deck = _deck(1)
    pl, _ = Q.deck_inputs(deck)
    ar, ai = _envelope(deck)
    mixed = Q.Simulation(deck.nr, deck.nz, 1, deck.dr, deck.dxi, precision=K.PREC_MIXED)
    with pytest.raises(Q.api.QpadError):
        mixed.add_laser(ar, ai, k0=K0)
    with pytest.raises(Q.api.QpadError):
        mixed.add_species(*pl, push_type=K.PUSH2_ROBUST_PGC)
    mixed.close()
    odd = Q.Simulation(48, deck.nz, 1, deck.dr, deck.dxi)
    with pytest.raises(Q.api.QpadError):
        odd.add_laser(np.zeros((deck.nz, 3, 48)), np.zeros((deck.nz, 3, 48)), k0=K0)
    odd.close()
