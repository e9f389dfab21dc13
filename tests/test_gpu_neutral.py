"""GPU parity of the ionising neutral gas (neutral_class.f03) against the CPU oracle.

One 3D step of a deck whose beam ionises a two-level gas: the per-slice iteration counts, the
3D stores, the electrons born (count exact, multiset) and the ionisation state per (angle,
cell) after the last slice.  Refusals: the mixed path, smoothing and the batched step.
"""
import numpy as np
import pytest

import qpad_gb300 as Q
from qpad_gb300 import _capi as K
from tests.helpers import sorted_rows, store_errors
from tests.test_neutral_cpu import _deck, neutral_spec, oracle_run

pytestmark = pytest.mark.gpu


def _gpu_sim(deck, pl, beams, spec, precision=K.PREC_FP64, smooth=0):
    sim = Q.Simulation(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi, iter_max=deck.iter_max,
                       iter_reltol=deck.iter_reltol, dt=deck.dt, precision=precision)
    if smooth:
        sim.set_smooth(smooth)
    sim.add_species(*pl)
    for bx, bp, bq in beams:
        sim.add_beam(bx, bp, bq)
    return sim


def test_ionising_gas_matches_oracle():
    deck = _deck()
    pl, beams = Q.deck_inputs(deck)
    spec = neutral_spec()
    osim, oiters = oracle_run(deck, pl, beams, spec)
    sim = _gpu_sim(deck, pl, beams, spec)
    gas = sim.add_neutral(spec["adk"], wp=spec["wp"], density=spec["density"], ppc=spec["ppc"],
                          num_theta=spec["num_theta"], qm=spec["qm"], qbm=spec["qbm"],
                          push_type=spec["push_type"], npmax=spec["npmax"])
    iters, _ = sim.run_3d_step()
    assert np.array_equal(iters, oiters), (iters, oiters)
    worst = {}
    for name in ("e", "b", "psi", "cu", "q_spe", "b_spe"):
        ref = osim.store(name)[:deck.nz]
        got = np.stack([sim.fields[name].store(s) for s in range(1, deck.nz + 1)])
        worst[name] = store_errors(got, ref).max()
    assert max(worst.values()) < 1e-9, worst
    # the ionisation state: fractions to round-off, the quantised mean exactly
    omi, mi = osim.multi_ion(), gas.ionisation_state()
    np.testing.assert_allclose(mi[:, :, :-1], omi[:, :, :-1], rtol=1e-9, atol=1e-12)
    assert np.array_equal(mi[:, :, -1], omi[:, :, -1])
    # the electrons born during the step, pushed to its end
    one = osim.neutral_plasma()
    x, p, g, ps, q = gas.download()
    assert one.n > 0 and len(q) == one.n
    np.testing.assert_allclose(sorted_rows(q, x[:, 0], x[:, 1]), sorted_rows(one.q, one.x, one.y),
                               rtol=1e-9, atol=1e-11)
    sim.close()


def test_neutral_gas_refusals():
    deck = _deck()
    pl, beams = Q.deck_inputs(deck)
    spec = neutral_spec()
    kw = dict(wp=spec["wp"], density=spec["density"], ppc=spec["ppc"], num_theta=spec["num_theta"])
    for precision, smooth in ((K.PREC_MIXED, 0), (K.PREC_FP64, 1)):
        sim = _gpu_sim(deck, pl, beams, spec, precision=precision, smooth=smooth)
        with pytest.raises(Q.api.QpadError):
            sim.add_neutral(spec["adk"], **kw)
        sim.close()
    sim = _gpu_sim(deck, pl, beams, spec)
    sim.add_neutral(spec["adk"], **kw)
    with pytest.raises(Q.api.QpadError):
        sim.set_smooth(1)
    sim.close()
