"""GPU parity of the fused slice loop (one 3D step) against the CPU oracle.

Same seeded plasma and beams go to both; the comparison covers the per-slice
predictor-corrector iteration counts, every slice of the 3D stores the step writes, the
surviving plasma particles (count exact, multiset) and the pushed beam.
"""
import numpy as np
import pytest

import qpad_gb300 as Q
from oracle import oracle as O
from tests.helpers import beam_to_oracle, field_errors, plasma_to_oracle, sorted_rows, store_errors

pytestmark = pytest.mark.gpu


def _deck(M, push_type=O.PUSH_ROBUST, nr=64):
    d = Q.decks.Deck("loop_test", nr=nr, nz=40, max_mode=M, dr=0.04, dxi=0.04, ppc=(2, 1), num_theta=8,
                     uth=2e-3, seed=3, beams=[Q.decks.BeamSpec(2.0, 0.4, 0.3, 0.6, 20000, x0=0.04)],
                     iter_max=30, iter_reltol=1e-6)
    return d


def _oracle_run(deck, pl_in, beams_in, push_type):
    g = O.grid(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi)
    x, p, gam, ps, q = pl_in
    sim = O.Sim(g, iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, iter_abstol=deck.iter_abstol,
                dt3d=deck.dt, sp_push_type=push_type, sp_npmax=len(q),
                beams=[(-1.0, O.PUSH3_REDUCED, len(b[2])) for b in beams_in])
    sim.set_plasma(plasma_to_oracle(x, p, gam, ps, q))
    for k, (bx, bp, bq) in enumerate(beams_in):
        sim.set_beam(k, beam_to_oracle(bx, bp, bq))
    iters, rel = sim.run_3dstep()
    return sim, iters, rel


# nr = 45 (one CTA of 45 rows) and nr = 66 (two CTAs of 33 rows) stage with 8-byte copies:
# the bulk-copy staging needs every row 16-byte aligned (even nr and rows per CTA)
@pytest.mark.parametrize("M,push_type,nr", [(1, O.PUSH_ROBUST, 64), (2, O.PUSH_ROBUST, 64), (2, O.PUSH_STD, 64),
                                            (2, O.PUSH_ROBUST, 45), (1, O.PUSH_STD, 66)])
def test_3d_step_matches_oracle(M, push_type, nr):
    deck = _deck(M, nr=nr)
    inputs = Q.deck_inputs(deck)
    pl, beams = inputs
    osim, oiters, orel = _oracle_run(deck, pl, beams, push_type)
    sim = Q.Simulation(deck.nr, deck.nz, M, deck.dr, deck.dxi, iter_max=deck.iter_max,
                       iter_reltol=deck.iter_reltol, dt=deck.dt)
    sim.add_species(*pl, push_type=push_type)
    for bx, bp, bq in beams:
        sim.add_beam(bx, bp, bq)
    iters, rel = sim.run_3d_step()
    # predictor-corrector iteration counts per slice (a metric of the path)
    assert np.array_equal(iters, oiters), (iters, oiters)
    worst = {}
    for name in ("e", "b", "psi", "cu", "q_spe", "b_spe", "e_spe", "q_beam"):
        ref = osim.store(name)[:deck.nz]
        got = np.stack([sim.fields[name].store(s) for s in range(1, deck.nz + 1)])
        worst[name] = store_errors(got, ref).max()
    assert max(worst.values()) < 1e-9, worst
    # plasma after the last slice: count exact, same particles
    opl = osim.plasma()
    x, p, g, ps, q = sim.species[0].download()
    assert len(q) == opl.n
    a = sorted_rows(q, x[:, 0], x[:, 1])
    b = sorted_rows(opl.q, opl.x, opl.y)
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-11)
    # beam after its push
    ob = osim.beam(0)
    bx, bp, bq = sim.beams[0].download()
    assert len(bq) == ob.n
    a = sorted_rows(bx[:, 2], bx[:, 0], bp[:, 0])
    b = sorted_rows(ob.z, ob.x, ob.px)
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12)
    sim.close()


@pytest.mark.parametrize("precision", [Q._capi.PREC_FP64, Q._capi.PREC_MIXED])
def test_graph_and_host_driven_loops_agree(precision):
    """The CUDA-graph slice loop (device-side WHILE conditions) equals the host-driven one."""
    deck = _deck(2)
    pl, beams = Q.deck_inputs(deck)
    runs = []
    for graph in (True, False):
        s = Q.Simulation(deck.nr, deck.nz, 2, deck.dr, deck.dxi, iter_max=deck.iter_max, dt=deck.dt,
                         precision=precision)
        s.lib.qpad_set_graph(s.h, int(graph))
        s.add_species(*pl)
        s.add_beam(*beams[0])
        it, _ = s.run_3d_step()
        import ctypes
        a = ctypes.c_int()
        s.lib.qpad_graph_active(s.h, ctypes.byref(a))
        assert a.value == int(graph)
        runs.append((it, [s.e.store(j) for j in (1, deck.nz // 2, deck.nz)], s))
    (ia, ea, sa), (ib, eb, sb) = runs
    if precision == Q._capi.PREC_FP64:
        assert np.array_equal(ia, ib)
        for x, y in zip(ea, eb):
            assert field_errors(x, y).max() < 1e-12
    else:
        # FP32 atomics make the two runs differ in summation order only; components far below
        # the field (E_phi of m = 0) are rated against 1e-3 of the field's norm
        assert abs(float(ia.mean()) - float(ib.mean())) < 0.5
        for x, y in zip(ea, eb):
            assert field_errors(x, y, floor_rel=1e-3).max() < 1e-4
    sa.close()
    sb.close()


def test_slice_by_slice_api_matches_fused_step():
    """qpad_slice_step driven from the host equals the fused 3D step."""
    deck = _deck(1)
    pl, beams = Q.deck_inputs(deck)
    a = Q.Simulation(deck.nr, deck.nz, 1, deck.dr, deck.dxi, iter_max=deck.iter_max, dt=deck.dt)
    a.add_species(*pl)
    a.add_beam(*beams[0])
    ia, _ = a.run_3d_step(push_beams=False)
    b = Q.Simulation(deck.nr, deck.nz, 1, deck.dr, deck.dxi, iter_max=deck.iter_max, dt=deck.dt)
    b.add_species(*pl)
    bm = b.add_beam(*beams[0])
    b.q_beam.store_fill(0.0)
    bm.qdp(b.q_beam)
    for f in ("b", "e", "b_spe", "e_spe", "psi", "cu", "acu", "amu"):
        b.fields[f].fill(0.0)
    ib = [b.slice_step(j).iters for j in range(1, deck.nz + 1)]
    assert list(ia) == ib
    for s in (1, deck.nz // 2, deck.nz):
        assert field_errors(b.e.store(s), a.e.store(s)).max() < 1e-12
    a.close()
    b.close()


@pytest.mark.parametrize("order", [1, 2])
def test_extrapolated_guess_matches_oracle(order):
    """The optional initial B-perp guess extrapolated from the previous slices (no counterpart
    in the reference; restated in the oracle): identical per-slice iteration counts and every
    store within 1e-9 on the FP64 path."""
    deck = _deck(2)
    pl, beams = Q.deck_inputs(deck)
    g = O.grid(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi)
    osim = O.Sim(g, iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, dt3d=deck.dt, sp_npmax=len(pl[4]),
                 beams=[(-1.0, O.PUSH3_REDUCED, len(beams[0][2]))], extrap=order)
    osim.set_plasma(plasma_to_oracle(*pl))
    osim.set_beam(0, beam_to_oracle(*beams[0]))
    oiters, _ = osim.run_3dstep()
    sim = Q.Simulation(deck.nr, deck.nz, 2, deck.dr, deck.dxi, iter_max=deck.iter_max,
                       iter_reltol=deck.iter_reltol, dt=deck.dt)
    sim.set_guess_extrapolation(order)
    sim.add_species(*pl)
    sim.add_beam(*beams[0])
    iters, _ = sim.run_3d_step()
    assert np.array_equal(iters, oiters), (iters, oiters)
    worst = {n: float(store_errors(sim.fields[n].store_all(), osim.store(n)[:deck.nz]).max())
             for n in ("e", "b", "psi", "cu", "b_spe")}
    assert max(worst.values()) < 1e-9, worst
    with pytest.raises(Q.QpadError):
        sim.set_guess_extrapolation(3)
    sim.close()


@pytest.mark.parametrize("unroll,iter_max", [(1, 30), (3, 30), (4, 30), (2, 3), (3, 4)])
def test_graph_unroll_matches_oracle(unroll, iter_max):
    """Iterations per body of the graph's iteration loop (the later ones return at once when
    the loop ended before them): identical per-slice iteration counts and stores within 1e-9
    of the oracle, also when the loop stops at iter_max inside a body."""
    deck = _deck(2)
    deck.iter_max = iter_max
    pl, beams = Q.deck_inputs(deck)
    osim, oiters, _ = _oracle_run(deck, pl, beams, O.PUSH_ROBUST)
    sim = Q.Simulation(deck.nr, deck.nz, 2, deck.dr, deck.dxi, iter_max=deck.iter_max,
                       iter_reltol=deck.iter_reltol, dt=deck.dt)
    sim.set_graph_unroll(unroll)
    sim.add_species(*pl)
    sim.add_beam(*beams[0])
    iters, _ = sim.run_3d_step()
    assert sim.graph_active()[0]
    assert np.array_equal(iters, oiters), (iters, oiters)
    worst = {n: float(store_errors(sim.fields[n].store_all(), osim.store(n)[:deck.nz]).max())
             for n in ("e", "b", "psi", "cu", "b_spe")}
    assert max(worst.values()) < 1e-9, worst
    with pytest.raises(Q.QpadError):
        sim.set_graph_unroll(5)
    sim.close()


def test_graph_unroll_mixed_path():
    """The mixed path with 1 and 3 iterations per loop body: the same iteration counts to
    within the FP32 atomics' summation order, fields within 1e-4."""
    deck = _deck(2)
    pl, beams = Q.deck_inputs(deck)
    runs = []
    for unroll in (1, 3):
        s = Q.Simulation(deck.nr, deck.nz, 2, deck.dr, deck.dxi, iter_max=deck.iter_max, dt=deck.dt,
                         precision=Q._capi.PREC_MIXED)
        s.set_graph_unroll(unroll)
        s.add_species(*pl)
        s.add_beam(*beams[0])
        it, _ = s.run_3d_step()
        runs.append((it, [s.e.store(j) for j in (1, deck.nz // 2, deck.nz)], s))
    (ia, ea, sa), (ib, eb, sb) = runs
    assert abs(float(ia.mean()) - float(ib.mean())) < 0.5
    for x, y in zip(ea, eb):
        assert field_errors(x, y, floor_rel=1e-3).max() < 1e-4
    sa.close()
    sb.close()
