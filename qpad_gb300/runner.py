"""Builds a Simulation from a synthetic deck (simulation::new for the benchmark shapes)."""
from __future__ import annotations

import numpy as np

from . import _capi as K
from .api import Simulation, load_beam, load_plasma
from .decks import Deck


def deck_inputs(deck: Deck, step: int = 0):
    """Host arrays of the plasma (for 3D step `step`) and of every beam, from the deck's seed.

    Plasma momenta are drawn from stream seed*1000 + step so that each 3D step's renewal is
    reproducible on its own; beams are drawn once from stream seed*1000 + 999 + k.
    """
    pl = load_plasma(deck.nr, deck.dr, deck.seed * 1000 + step, deck.ppc[0], deck.ppc[1], deck.num_theta,
                     uth=(deck.uth, deck.uth, deck.uth))
    beams = []
    for k, b in enumerate(deck.beams):
        args = b.load_args(deck.nz, deck.dxi)
        if args["range_lo"][2] >= args["range_hi"][2]:       # beam entirely behind a shortened box
            beams.append((np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0)))
            continue
        beams.append(load_beam(deck.nr, deck.nz, deck.dr, deck.dxi, deck.seed * 1000 + 999 + k, **args))
    return pl, beams


def build_simulation(deck: Deck, precision=K.PREC_FP64, device=0, sort_freq=0, inputs=None) -> Simulation:
    sim = Simulation(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi, iter_max=deck.iter_max,
                     iter_reltol=deck.iter_reltol, iter_abstol=deck.iter_abstol, dt=deck.dt, precision=precision,
                     device=device)
    if deck.smooth_order:
        sim.set_smooth(deck.smooth_order)
    pl, beams = inputs if inputs is not None else deck_inputs(deck)
    x, p, g, ps, q = pl
    sim.add_species(x, p, g, ps, q, qbm=-1.0, npmax=max(1, len(q)), sort_freq=sort_freq)
    for (bx, bp, bq), spec in zip(beams, deck.beams):
        sim.add_beam(bx, bp, bq, qbm=spec.qm, npmax=max(1, len(bq)))
    return sim
