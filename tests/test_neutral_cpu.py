"""Neutral gas on the CPU: the ADK coefficients against the formula worked by hand for
hydrogen, and the oracle's ionisation bookkeeping (neutral_class.f03:576-878)."""
import math

import numpy as np

import qpad_gb300 as Q
from oracle import oracle as O
from qpad_gb300.neutrals import E_A_GVM, OMEGA_A, adk_coefficients, plasma_frequency
from tests.helpers import beam_to_oracle, plasma_to_oracle


def test_adk_hydrogen_by_hand():
    # U = 1/2 hartree, n* = 1, C^2 = 2^2 / (1 * 1 * 1) = 4:
    # p1 = omega_a * 4 * 0.5 * (2 E_a), p2 = 2 E_a / 3, p3 = 1
    (p1, p2, p3), = adk_coefficients([0.5 * 27.211386245988])
    assert math.isclose(p3, 1.0, rel_tol=1e-12)
    assert math.isclose(p2, 2.0 * E_A_GVM / 3.0, rel_tol=1e-12)
    assert math.isclose(p1, OMEGA_A * 4.0 * 0.5 * 2.0 * E_A_GVM, rel_tol=1e-12)


def _deck():
    return Q.decks.Deck("neut", nr=40, nz=20, max_mode=1, dr=0.05, dxi=0.05, ppc=(2, 1), num_theta=8, uth=0.0,
                        seed=6, beams=[Q.decks.BeamSpec(6.0, 0.3, 0.3, 0.45, 20000, x0=0.02)], iter_max=20)


def neutral_spec():
    # hydrogen-like first level and a second at 24.6 eV, a gas of 1e18 cm^-3: both levels partly ionise
    return dict(adk=adk_coefficients([13.6, 24.6]), wp=plasma_frequency(1e18), density=0.5, ppc=(2, 1),
                num_theta=8, qm=-1.0, qbm=-1.0, push_type=O.PUSH_ROBUST, npmax=40 * 2 * 8 * 2 + 64)


def oracle_run(deck, pl, beams, neutral):
    g = O.grid(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi)
    sim = O.Sim(g, iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, dt3d=deck.dt, sp_npmax=len(pl[4]),
                beams=[(-1.0, O.PUSH3_REDUCED, len(b[2])) for b in beams], neutral=neutral)
    sim.set_plasma(plasma_to_oracle(*pl))
    for k, b in enumerate(beams):
        sim.set_beam(k, beam_to_oracle(*b))
    its, _ = sim.run_3dstep()
    return sim, its


def test_oracle_ionisation_bookkeeping():
    deck = _deck()
    (pl, beams), spec = Q.deck_inputs(deck), neutral_spec()
    sim, _ = oracle_run(deck, pl, beams, spec)
    mi = sim.multi_ion()
    L, ppc_tot = 2, 2
    frac = mi[:, :, :L + 1]
    assert np.all(frac >= -1e-15) and np.all(frac <= 1.0 + 1e-15)
    assert np.all(np.abs(frac.sum(axis=2) - 1.0) < 1e-12)          # levels + neutral fraction
    q = mi[:, :, L + 1] * ppc_tot / L                                # the quantised mean, in electrons
    assert np.allclose(q, np.round(q))
    assert q.sum() > 0, "the deck ionises"
    # every electron born is still in the box: one per quantum of the mean ionisation
    assert sim.neutral_plasma().n == int(round(q.sum()))
