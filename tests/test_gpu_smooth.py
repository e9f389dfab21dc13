"""Binomial smoothing of the species deposits against the CPU oracle, which applies
ufield::smooth_f1 smooth_order times: the per-op charge and current deposits, and whole 3D
steps through the fused loop (orders 1-2 inside the iteration kernel's node window, higher
orders as a pass of their own before it)."""
import numpy as np
import pytest

import qpad_gb300 as Q
from oracle import oracle as O
from tests.helpers import field_errors, plasma_to_oracle, smooth_field, store_errors

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _plasma(nr, dr, seed):
    x, p, g, ps, q = Q.load_plasma(nr, dr, seed, 2, 2, 8, uth=(0.05, 0.05, 0.05))
    rng = np.random.default_rng(seed)
    x = np.ascontiguousarray(x + rng.uniform(-0.45, 0.45, x.shape) * dr)
    ps = np.ascontiguousarray(rng.uniform(-0.2, 0.2, len(q)))
    return x, p, g, ps, q


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("nr,M", [(64, 1), (96, 3)])
def test_qdp_smoothed(order, nr, M):
    dr = 0.04
    g = O.grid(nr, 4, M, dr, 0.04)
    sim = Q.Simulation(nr, 4, M, dr, 0.04)
    sim.set_smooth(order)
    x, p, gam, ps, q = _plasma(nr, dr, nr + M)
    sp = sim.add_species(x, p, gam, ps, q, neutralized=False)
    sim.q_spe.fill(0.0)
    sp.qdp(sim.q_spe)
    ref = O.qdeposit(g, plasma_to_oracle(x, p, gam, ps, q))
    for _ in range(order):
        O.smooth(g, 0, ref)
    assert field_errors(sim.q_spe.download(), ref, nodes=slice(0, None)).max() < TOL
    sim.close()


@pytest.mark.parametrize("order", [1, 2, 4])
@pytest.mark.parametrize("push_type", [O.PUSH_ROBUST, O.PUSH_STD])
def test_amjdp_smoothed(order, push_type):
    nr, M, dr, dt = 96, 2, 0.04, 0.04
    g = O.grid(nr, 4, M, dr, dt)
    rng = np.random.default_rng(7 + order + push_type)
    ef = smooth_field(rng, g, 3, scale=0.5)
    bf = smooth_field(rng, g, 3, scale=0.5)
    sim = Q.Simulation(nr, 4, M, dr, dt)
    sim.set_smooth(order)
    x, p, gam, ps, q = _plasma(nr, dr, 11)
    sp = sim.add_species(x, p, gam, ps, q, push_type=push_type)
    sim.e.upload(ef)
    sim.b.upload(bf)
    for f in (sim.cu, sim.amu, sim.acu):
        f.fill(0.0)
    sp.amjdp(sim.e, sim.b, sim.cu, sim.amu, sim.acu, dt)
    cu, amu, dcu = O.amjdeposit(g, push_type, -1.0, dt, plasma_to_oracle(x, p, gam, ps, q), ef, bf)
    for _ in range(order):
        O.smooth(g, 1, cu)
        O.smooth(g, 2, dcu)
        O.smooth(g, 1, amu)
    assert field_errors(sim.cu.download(), cu, nodes=slice(0, None)).max() < TOL
    assert field_errors(sim.amu.download(), amu, nodes=slice(0, None)).max() < TOL
    assert field_errors(sim.acu.download(), dcu, nodes=slice(0, None)).max() < TOL
    sim.close()


def test_smooth_order_limits():
    sim = Q.Simulation(32, 4, 1, 0.04, 0.04)
    with pytest.raises(Q.QpadError):
        sim.set_smooth(65)
    with pytest.raises(Q.QpadError):
        sim.set_smooth(-1)
    sim.set_smooth(64)
    sim.set_smooth(2)
    sim.set_smooth(0)
    sim.close()


# (nr 66: two CTAs of 33 rows, the 8-byte staging path)
@pytest.mark.parametrize("order,M,push_type,nr", [(1, 2, O.PUSH_ROBUST, 64), (2, 1, O.PUSH_STD, 64),
                                                  (2, 2, O.PUSH_ROBUST, 66), (3, 2, O.PUSH_ROBUST, 64),
                                                  (5, 1, O.PUSH_STD, 66)])
def test_3d_step_smoothed_matches_oracle(order, M, push_type, nr):
    deck = Q.decks.Deck("smooth_loop", nr=nr, nz=32, max_mode=M, dr=0.04, dxi=0.04, ppc=(2, 1), num_theta=8,
                        uth=2e-3, seed=5, beams=[Q.decks.BeamSpec(2.0, 0.4, 0.3, 0.6, 20000, x0=0.04)],
                        iter_max=30, iter_reltol=1e-6, smooth_order=order)
    pl, beams = Q.deck_inputs(deck)
    g = O.grid(deck.nr, deck.nz, M, deck.dr, deck.dxi)
    x, p, gam, ps, q = pl
    osim = O.Sim(g, iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, iter_abstol=deck.iter_abstol,
                 dt3d=deck.dt, sp_push_type=push_type, sp_npmax=len(q),
                 beams=[(-1.0, O.PUSH3_REDUCED, len(b[2])) for b in beams], smooth_order=order)
    osim.set_plasma(plasma_to_oracle(x, p, gam, ps, q))
    from tests.helpers import beam_to_oracle
    for k, (bx, bp, bq) in enumerate(beams):
        osim.set_beam(k, beam_to_oracle(bx, bp, bq))
    oiters, _ = osim.run_3dstep()
    sim = Q.Simulation(deck.nr, deck.nz, M, deck.dr, deck.dxi, iter_max=deck.iter_max,
                       iter_reltol=deck.iter_reltol, dt=deck.dt)
    sim.set_smooth(order)
    sim.add_species(*pl, push_type=push_type)
    for bx, bp, bq in beams:
        sim.add_beam(bx, bp, bq)
    iters, _ = sim.run_3d_step()
    assert np.array_equal(iters, oiters), (iters, oiters)
    worst = {}
    for name in ("e", "b", "psi", "cu", "q_spe", "b_spe"):
        ref = osim.store(name)[:deck.nz]
        got = np.stack([sim.fields[name].store(s) for s in range(1, deck.nz + 1)])
        worst[name] = store_errors(got, ref).max()
    assert max(worst.values()) < 1e-9, worst
    sim.close()


def test_mixed_step_smoothed_close_to_fp64():
    deck = Q.decks.Deck("smooth_mixed", nr=64, nz=24, max_mode=2, dr=0.04, dxi=0.04, ppc=(2, 1), num_theta=8,
                        uth=2e-3, seed=6, beams=[Q.decks.BeamSpec(2.0, 0.4, 0.3, 0.5, 20000, x0=0.04)],
                        iter_max=30, iter_reltol=1e-6, smooth_order=1)
    inputs = Q.deck_inputs(deck)
    a = Q.build_simulation(deck, precision=Q._capi.PREC_FP64, inputs=inputs)
    b = Q.build_simulation(deck, precision=Q._capi.PREC_MIXED, inputs=inputs)
    a.run_3d_step()
    b.run_3d_step()
    for f in ("e", "b"):
        ga = np.stack([a.fields[f].store(s) for s in range(1, deck.nz + 1)])
        gb = np.stack([b.fields[f].store(s) for s in range(1, deck.nz + 1)])
        assert store_errors(gb, ga).max() < 1e-3, f
    a.close()
    b.close()
