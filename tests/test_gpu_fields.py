"""GPU parity of the per-mode field solves against the CPU oracle (FP64, 1e-10 rel L2).

Each case fills the source fields with seeded smooth random profiles, runs the reference
routine in the oracle and the same routine through the C ABI, and compares every mode
part and component over nodes 1..nr.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import field_errors, smooth_field

TOL = 1e-10   # plain FP64 path: only summation / FMA order differs

pytestmark = pytest.mark.gpu

CASES = [(64, 1, 0.04), (256, 2, 0.02), (512, 4, 0.01), (100, 3, 0.05)]


def _sim(nr, M, dr, bnd=O.BND_OPEN):
    import qpad_gb300 as Q
    return Q.Simulation(nr, 4, M, dr, 0.02, bnd=bnd)


@pytest.mark.parametrize("nr,M,dr", CASES)
@pytest.mark.parametrize("bnd", [O.BND_OPEN, O.BND_ZERO])
def test_psi_bz_ez_bt_beam(nr, M, dr, bnd):
    rng = np.random.default_rng(nr * 10 + M)
    g = O.grid(nr, 4, M, dr, 0.02, bnd=bnd)
    sim = _sim(nr, M, dr, bnd)
    q = smooth_field(rng, g, 1)
    cu = smooth_field(rng, g, 3, zero_guards=False)
    sim.q_spe.upload(q)
    sim.cu.upload(cu)
    sim.q_beam.upload(q)
    sim.psi.solve(sim.q_spe)
    assert field_errors(sim.psi.download(), O.solve_psi(g, q)).max() < TOL
    sim.b_spe.fill(0.0)
    sim.b_spe.solve(sim.cu)
    assert field_errors(sim.b_spe.download(), O.solve_bz(g, cu)).max() < TOL
    sim.e.fill(0.0)
    sim.e.solve(sim.cu)
    assert field_errors(sim.e.download(), O.solve_ez(g, cu)).max() < TOL
    sim.b_beam.fill(0.0)
    sim.b_beam.solve(sim.q_beam)
    assert field_errors(sim.b_beam.download(), O.solve_bt_beam(g, q)).max() < TOL
    sim.close()


@pytest.mark.parametrize("nr,M,dr", CASES)
def test_bt_iter_et_djdxi(nr, M, dr):
    rng = np.random.default_rng(nr * 7 + M)
    g = O.grid(nr, 4, M, dr, 0.02)
    sim = _sim(nr, M, dr)
    dcu = smooth_field(rng, g, 2)
    cu = smooth_field(rng, g, 3, zero_guards=False)
    b0 = smooth_field(rng, g, 3)
    psi = smooth_field(rng, g, 1)
    acu = smooth_field(rng, g, 2, zero_guards=False)
    amu = smooth_field(rng, g, 3, zero_guards=False)
    sim.dcu.upload(dcu)
    sim.cu.upload(cu)
    sim.b_spe.upload(b0)
    sim.b_spe.solve(sim.dcu, sim.cu)
    ref = O.solve_bt_iter(g, dcu, cu, b0.copy())
    assert field_errors(sim.b_spe.download(), ref).max() < TOL
    sim.b.upload(b0)
    sim.psi.upload(psi)
    sim.e.fill(0.0)
    sim.e.solve(sim.b, sim.psi)
    assert field_errors(sim.e.download(), O.solve_et(g, b0, psi)).max() < TOL
    sim.acu.upload(acu)
    sim.amu.upload(amu)
    sim.dcu.fill(0.0)
    sim.dcu.solve(sim.acu, sim.amu)
    assert field_errors(sim.dcu.download(), O.solve_djdxi(g, acu, amu)).max() < TOL
    sim.close()


@pytest.mark.parametrize("nr,M,dr", CASES[:3])
def test_conv_test(nr, M, dr):
    rng = np.random.default_rng(3 + M)
    g = O.grid(nr, 4, M, dr, 0.02)
    sim = _sim(nr, M, dr)
    b_old = smooth_field(rng, g, 3)
    b_new = b_old + 1e-5 * smooth_field(rng, g, 3)
    sim.b_spe.upload(b_old)
    sim.conv_test(sim.b_spe, "record")
    sim.b_spe.upload(b_new)
    rel, ab = sim.conv_test(sim.b_spe, "compare")
    rel_o, ab_o = O.conv_test(g, b_old, b_new)
    assert abs(rel - rel_o) <= 1e-12 * rel_o
    assert abs(ab - ab_o) <= 1e-12 * ab_o
    sim.close()


def test_field_arithmetic_and_slices():
    import qpad_gb300 as Q
    rng = np.random.default_rng(11)
    g = O.grid(64, 6, 2, 0.04, 0.04)
    sim = Q.Simulation(64, 6, 2, 0.04, 0.04)
    a, b = smooth_field(rng, g, 3), smooth_field(rng, g, 3)
    sim.b_spe.upload(a)
    sim.b_beam.upload(b)
    Q.add_f1(sim.b_spe, sim.b_beam, sim.b)
    assert np.array_equal(sim.b.download(), a + b)
    sim.cu.upload(a)
    q = smooth_field(rng, g, 1)
    sim.q_spe.upload(q)
    Q.add_f1_dim(sim.cu, sim.q_spe, [3], [1])
    expect = q.copy()
    expect[:, 0] += a[:, 2]
    assert np.array_equal(sim.q_spe.download(), expect)
    sim.cu.scale(0.5)
    assert np.array_equal(sim.cu.download(), a * 0.5)
    sim.e.upload(b)
    sim.e.copy_slice(3, Q._capi.COPY_1TO2)
    assert np.array_equal(sim.e.store(3), b)
    sim.e.fill(0.0)
    sim.e.copy_slice(3, Q._capi.COPY_2TO1)
    assert np.array_equal(sim.e.download(), b)
    sim.close()


def test_species_cbq():
    """cbq_species2d (species2d_class.f03:396-410): q(1) += cu(3), then q's slice into its store;
    the store read in one copy returns the same slices."""
    import qpad_gb300 as Q
    rng = np.random.default_rng(12)
    nr, M, nz = 48, 2, 6
    g = O.grid(nr, nz, M, 0.05, 0.05)
    sim = Q.Simulation(nr, nz, M, 0.05, 0.05)
    x, p, gam, ps, qq = Q.load_plasma(nr, 0.05, 3, 1, 1, 8)
    sp = sim.add_species(x, p, gam, ps, qq)
    sim.q_spe.store_fill(0.0)
    expect = {}
    for pos in (1, 4, nz):
        q = smooth_field(rng, g, 1)
        cu = smooth_field(rng, g, 3, zero_guards=False)
        sim.q_spe.upload(q)
        sim.cu.upload(cu)
        sp.cbq(pos, sim.q_spe, sim.cu)
        want = q.copy()
        want[:, 0] += cu[:, 2]
        assert np.array_equal(sim.q_spe.download(), want)
        assert np.array_equal(sim.q_spe.store(pos), want)
        expect[pos] = want
    allq = sim.q_spe.store_all()
    assert allq.shape == (nz, 2 * M + 1, 1, nr + 2)
    for pos, want in expect.items():
        assert np.array_equal(allq[pos - 1], want)
    assert np.count_nonzero(allq[1]) == 0
    with pytest.raises(Q.QpadError):
        sp.cbq(nz + 2, sim.q_spe, sim.cu)
    with pytest.raises(Q.QpadError):
        sp.cbq(1, sim.cu, sim.q_spe)
    sim.close()
