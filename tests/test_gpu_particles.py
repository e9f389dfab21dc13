"""GPU parity of the plasma and beam particle kernels against the CPU oracle.

Deposits and pushes are FP64 and must agree within 1e-10 relative L2 (summation order of
the atomics differs); cell keys, the sort permutation and particle counts are integer
work and must agree exactly.
"""
import numpy as np
import pytest

import qpad_gb300 as Q
from oracle import oracle as O
from tests.helpers import beam_to_oracle, field_errors, plasma_to_oracle, smooth_field, sorted_rows

TOL = 1e-10
pytestmark = pytest.mark.gpu


def _plasma(nr, dr, seed, ppc=(2, 2), ntheta=8, uth=0.05, jitter=0.45):
    """Loaded plasma with jittered positions and thermal momenta (seeded)."""
    x, p, g, ps, q = Q.load_plasma(nr, dr, seed, ppc[0], ppc[1], ntheta, uth=(uth, uth, uth))
    rng = np.random.default_rng(seed)
    x = x + rng.uniform(-jitter, jitter, x.shape) * dr
    x = np.ascontiguousarray(x)
    ps = np.ascontiguousarray(rng.uniform(-0.2, 0.2, len(q)))
    return x, p, g, ps, q


@pytest.mark.parametrize("nr,M", [(64, 1), (128, 2), (96, 4)])
def test_qdeposit(nr, M):
    dr = 0.04
    g = O.grid(nr, 4, M, dr, 0.04)
    sim = Q.Simulation(nr, 4, M, dr, 0.04)
    x, p, gam, ps, q = _plasma(nr, dr, nr + M)
    sp = sim.add_species(x, p, gam, ps, q, neutralized=False)
    sim.q_spe.fill(0.0)
    sp.qdp(sim.q_spe)
    ref = O.qdeposit(g, plasma_to_oracle(x, p, gam, ps, q))
    assert field_errors(sim.q_spe.download(), ref, nodes=slice(0, None)).max() < TOL
    sim.close()


def test_neutralised_qdp_cancels():
    nr, M, dr = 64, 2, 0.04
    sim = Q.Simulation(nr, 4, M, dr, 0.04)
    x, p, gam, ps, q = _plasma(nr, dr, 5)
    sp = sim.add_species(x, p, gam, ps, q, neutralized=True)
    sim.q_spe.fill(0.0)
    sp.qdp(sim.q_spe)
    out = sim.q_spe.download()
    g = O.grid(nr, 4, M, dr, 0.04)
    scale = np.abs(O.qdeposit(g, plasma_to_oracle(x, p, gam, ps, q))).max()
    assert np.abs(out).max() <= 1e-13 * scale
    sim.close()


@pytest.mark.parametrize("push_type", [O.PUSH_ROBUST, O.PUSH_STD])
@pytest.mark.parametrize("nr,M", [(64, 1), (128, 2), (96, 4)])
def test_amjdp(push_type, nr, M):
    dr, dt = 0.04, 0.04
    g = O.grid(nr, 4, M, dr, dt)
    rng = np.random.default_rng(100 + nr + M + push_type)
    ef = smooth_field(rng, g, 3, scale=0.5)
    bf = smooth_field(rng, g, 3, scale=0.5)
    sim = Q.Simulation(nr, 4, M, dr, dt)
    x, p, gam, ps, q = _plasma(nr, dr, 7 + nr)
    sp = sim.add_species(x, p, gam, ps, q, push_type=push_type)
    sim.e.upload(ef)
    sim.b.upload(bf)
    for f in (sim.cu, sim.amu, sim.acu):
        f.fill(0.0)
    sp.amjdp(sim.e, sim.b, sim.cu, sim.amu, sim.acu, dt)
    pl = plasma_to_oracle(x, p, gam, ps, q)
    cu, amu, dcu = O.amjdeposit(g, push_type, -1.0, dt, pl, ef, bf)
    assert field_errors(sim.cu.download(), cu, nodes=slice(0, None)).max() < TOL
    assert field_errors(sim.amu.download(), amu, nodes=slice(0, None)).max() < TOL
    assert field_errors(sim.acu.download(), dcu, nodes=slice(0, None)).max() < TOL
    _, _, g2, ps2, _ = sp.download()
    np.testing.assert_allclose(g2, pl.gamma, rtol=1e-13)
    np.testing.assert_allclose(ps2, pl.psi, rtol=1e-12, atol=1e-14)
    sim.close()


@pytest.mark.parametrize("push_type", [O.PUSH_ROBUST, O.PUSH_STD])
@pytest.mark.parametrize("nr,M", [(64, 2), (128, 4)])
def test_push_u_push_x_update_bound(push_type, nr, M):
    dr, dt = 0.04, 0.2
    g = O.grid(nr, 4, M, dr, dt)
    rng = np.random.default_rng(200 + nr + M + push_type)
    ef = smooth_field(rng, g, 3, scale=2.0)
    bf = smooth_field(rng, g, 3, scale=2.0)
    sim = Q.Simulation(nr, 4, M, dr, dt)
    x, p, gam, ps, q = _plasma(nr, dr, 9 + nr, uth=0.3)
    sp = sim.add_species(x, p, gam, ps, q, push_type=push_type)
    sim.e.upload(ef)
    sim.b.upload(bf)
    sp.push_u(sim.e, sim.b, dt)
    pl = plasma_to_oracle(x, p, gam, ps, q)
    O.push_u(g, push_type, -1.0, dt, pl, ef, bf)
    x1, p1, g1, _, _ = sp.download()
    np.testing.assert_allclose(p1, np.stack([pl.px, pl.py, pl.pz], 1), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(g1, pl.gamma, rtol=1e-13)
    sp.push_x(dt)
    O.push_x(pl, dt)
    n = O.update_bound(g, pl)
    assert n < len(q), "the case must remove some particles at the edge"
    assert sp.count() == n                                   # particle count is bit-exact
    x2, p2, g2, ps2, q2 = sp.download()
    a = sorted_rows(q2, x2[:, 0], x2[:, 1], p2[:, 2])
    b = sorted_rows(pl.q[:n], pl.x[:n], pl.y[:n], pl.pz[:n])
    np.testing.assert_array_equal(a[:, 0], b[:, 0])          # same particle set (by charge order)
    np.testing.assert_allclose(a, b, rtol=1e-11, atol=1e-13)
    sim.close()


@pytest.mark.parametrize("nr,M", [(64, 2), (256, 1)])
def test_interp_psi(nr, M):
    dr = 0.04
    g = O.grid(nr, 4, M, dr, 0.04)
    rng = np.random.default_rng(300 + nr)
    psif = smooth_field(rng, g, 1)
    sim = Q.Simulation(nr, 4, M, dr, 0.04)
    x, p, gam, ps, q = _plasma(nr, dr, 13)
    sp = sim.add_species(x, p, gam, ps, q, push_type=O.PUSH_STD)
    sim.psi.upload(psif)
    sp.interp_psi(sim.psi)
    pl = plasma_to_oracle(x, p, gam, ps, q)
    O.interp_psi(g, pl, psif)
    np.testing.assert_allclose(sp.download()[3], pl.psi, rtol=1e-12, atol=1e-14)
    sim.close()


@pytest.mark.parametrize("nr,ntheta", [(64, 8), (300, 4)])
def test_sort_matches_reference_permutation(nr, ntheta):
    dr = 0.03
    g = O.grid(nr, 4, 1, dr, 0.04)
    sim = Q.Simulation(nr, 4, 1, dr, 0.04)
    x, p, gam, ps, q = _plasma(nr, dr, 17, ntheta=ntheta, jitter=3.0)
    r = np.hypot(x[:, 0], x[:, 1])
    keep = r < nr * dr * 0.999
    x, p, gam, ps, q = (np.ascontiguousarray(a[keep]) for a in (x, p, gam, ps, q))
    sp = sim.add_species(x, p, gam, ps, q)
    sp.sort()
    pl = plasma_to_oracle(x, p, gam, ps, q)
    keys, idx = O.sort(g, pl)
    x2, p2, g2, ps2, q2 = sp.download()
    np.testing.assert_array_equal(x2[:, 0], pl.x)
    np.testing.assert_array_equal(x2[:, 1], pl.y)
    np.testing.assert_array_equal(p2, np.stack([pl.px, pl.py, pl.pz], 1))
    np.testing.assert_array_equal(q2, pl.q)
    np.testing.assert_array_equal(ps2, pl.psi)
    sim.close()


@pytest.mark.parametrize("nr,nz,M", [(64, 32, 1), (128, 40, 3)])
def test_beam_qdeposit(nr, nz, M):
    dr, dxi = 0.04, 0.05
    g = O.grid(nr, nz, M, dr, dxi)
    spec = Q.decks.BeamSpec(2.0, 0.4, 0.4, 1.0, 20000, x0=0.05)
    args = spec.load_args(nz, dxi)
    bx, bp, bq = Q.load_beam(nr, nz, dr, dxi, 21, **args)
    sim = Q.Simulation(nr, nz, M, dr, dxi)
    bm = sim.add_beam(bx, bp, bq)
    sim.q_beam.store_fill(0.0)
    bm.qdp(sim.q_beam)
    ref = O.beam_qdeposit(g, beam_to_oracle(bx, bp, bq))
    for s in range(1, nz + 2):
        got = sim.q_beam.store(s)
        assert field_errors(got, ref[s - 1], nodes=slice(0, None)).max() < TOL, s
    sim.close()


@pytest.mark.parametrize("push_type", [O.PUSH3_REDUCED, O.PUSH3_BORIS])
def test_beam_push(push_type):
    nr, nz, M, dr, dxi = 64, 24, 2, 0.04, 0.05
    g = O.grid(nr, nz, M, dr, dxi)
    rng = np.random.default_rng(400 + push_type)
    spec = Q.decks.BeamSpec(2.0, 0.6, 0.4, 1.0, 20000, eps_n=0.5)
    bx, bp, bq = Q.load_beam(nr, nz, dr, dxi, 23, **spec.load_args(nz, dxi))
    bp = np.ascontiguousarray(bp * np.array([1.0, 1.0, 1e-4]))   # slow beam: particles leave the box
    sim = Q.Simulation(nr, nz, M, dr, dxi, dt=0.5)
    bm = sim.add_beam(bx, bp, bq, push_type=push_type)
    e2, b2 = O.store(g, 3), O.store(g, 3)
    for s in range(1, nz + 1):
        e2[s - 1] = smooth_field(rng, g, 3)
        b2[s - 1] = smooth_field(rng, g, 3)
        sim.e.store_upload(s, e2[s - 1])
        sim.b.store_upload(s, b2[s - 1])
    bm.push(sim.e, sim.b)
    ob = beam_to_oracle(bx, bp, bq)
    O.beam_push(g, push_type, -1.0, 0.5, ob, e2, b2)
    n = O.beam_update_bound(g, ob)
    assert n < len(bq)
    assert bm.count() == n
    x2, p2, q2 = bm.download()
    a = sorted_rows(x2[:, 0], x2[:, 1], x2[:, 2], p2[:, 0], p2[:, 2])
    b = sorted_rows(ob.x[:n], ob.y[:n], ob.z[:n], ob.px[:n], ob.pz[:n])
    np.testing.assert_allclose(a, b, rtol=1e-11, atol=1e-12)
    sim.close()
