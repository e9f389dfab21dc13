"""Known-answer tests that pin the CPU oracle to the physics and to the reference's rules.

The reference's own tests hold no assertions or stored outputs, so the oracle is pinned
here instead: manufactured solutions of every tridiagonal operator kind (second-order
convergence to the continuous radial operator), hand-expanded deposits and pushes of
single particles, the exact permutations of update_bound and the counting sort, the
neutral-plasma invariant, and the linear-wake period.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


def _radial_operator_error(kind, m, nr, R=6.0, a=1.0):
    """Discrete solve of the (kind, m) operator applied to u = r^k exp(-r^2/a^2).

    k is the azimuthal order the operator carries (m for psi/Ez/Bz/beam Bt, m+1 for B+,
    |m-1| for B-).  For that u the continuous operator is exact in closed form:
    u'' + u'/r - k^2 u/r^2 = (4 r^(k+2)/a^4 - 4 (k+1) r^k/a^2) exp(-r^2/a^2),
    and the B+/B- operators subtract relax_fac/dr^2 (constant for the default relax_fac).
    """
    dr = R / nr
    g = O.grid(nr, 1, max(m, 1), dr, 0.02)
    A, B, Cc = O.build_matrix(g, kind, m)
    r = np.arange(nr) * dr                           # row k (node k+1) sits at r = k dr
    k = {O.FK_PSI: m, O.FK_BZ: m, O.FK_EZ: m, O.FK_BT: m, O.FK_BPLUS: m + 1, O.FK_BMINUS: abs(m - 1)}[kind]
    e = np.exp(-(r / a) ** 2)
    u = r ** k * e
    lap = (4 * r ** (k + 2) / a ** 4 - 4 * (k + 1) * r ** k / a ** 2) * e
    rf = g.relax_fac / dr ** 2 if kind in (O.FK_BPLUS, O.FK_BMINUS) else 0.0
    x = lap - rf * u
    if B[0] * dr ** 2 == 1.0:                        # identity axis row: u(0) = 0
        x[0] = 0.0
    x = np.ascontiguousarray(x)
    O.lib().orc_thomas(nr, O.ptr(A), O.ptr(B), O.ptr(Cc), O.ptr(x))
    return float(np.max(np.abs(x - u))) / float(np.max(np.abs(u)))


@pytest.mark.parametrize("kind,m", [(O.FK_PSI, 0), (O.FK_PSI, 1), (O.FK_PSI, 2), (O.FK_BZ, 3),
                                    (O.FK_BPLUS, 0), (O.FK_BPLUS, 1), (O.FK_BMINUS, 0), (O.FK_BMINUS, 1),
                                    (O.FK_BMINUS, 2)])
def test_operators_converge_second_order(kind, m):
    e1 = _radial_operator_error(kind, m, 96)
    e2 = _radial_operator_error(kind, m, 192)
    e3 = _radial_operator_error(kind, m, 384)
    assert e3 < 2e-3
    assert e1 / e2 > 3.0 and e2 / e3 > 3.0, (e1, e2, e3)


def test_matrix_rows_follow_field_solver():
    """Interior, axis and open-boundary rows of set_struct_matrix, written out by hand."""
    nr, dr = 16, 0.1
    g = O.grid(nr, 1, 2, dr, 0.1, relax_fac=0.01)
    a, b, c = O.build_matrix(g, O.FK_PSI, 2)
    j = 5.0
    assert a[5] * dr ** 2 == pytest.approx(1 - 0.5 / j) and c[5] * dr ** 2 == pytest.approx(1 + 0.5 / j)
    assert b[5] * dr ** 2 == pytest.approx(-2 - 4 / j ** 2)
    assert (a[0], b[0] * dr ** 2, c[0], a[1]) == (0.0, 1.0, 0.0, 0.0)            # decoupled axis, m > 0
    jm = 15.0
    assert b[-1] * dr ** 2 == pytest.approx(-2 - 4 / jm ** 2 + (1 - 2 / nr) * (1 + 0.5 / jm)) and c[-1] == 0.0
    a0, b0, c0 = O.build_matrix(g, O.FK_PSI, 0)
    assert (b0[0] * dr ** 2, c0[0] * dr ** 2) == (-4.0, 4.0)
    assert c0[-1] == 0.0 and b0[-1] * dr ** 2 == pytest.approx(-2.0)              # Dirichlet for m = 0
    ap, bp, cp = O.build_matrix(g, O.FK_BPLUS, 1)
    assert bp[5] * dr ** 2 == pytest.approx(-2 - (2 / j) ** 2 - 0.01)
    am, bm, cm = O.build_matrix(g, O.FK_BMINUS, 1)
    assert (bm[0] * dr ** 2, cm[0] * dr ** 2) == (pytest.approx(-4.01), pytest.approx(4.0))
    # B- outer row uses (m+1) like B+ (field_solver_class.f03:532-535)
    assert bm[-1] * dr ** 2 == pytest.approx(-2 - 0.01 + (1 - 2 / nr) * (1 + 0.5 / jm))
    at, bt, ct = O.build_matrix(g, O.FK_BT, 0)
    fac = 1 + 1 / (nr * math.log(nr * dr))
    assert bt[-1] * dr ** 2 == pytest.approx(-2 + fac * (1 + 0.5 / jm))


def test_single_particle_charge_deposit():
    nr, dr = 16, 0.1
    g = O.grid(nr, 1, 2, dr, 0.1)
    pl = O.Plasma(1)
    r, phi, f = (4 + 0.3) * dr, 0.7, 0.3
    pl.x[0], pl.y[0], pl.q[0] = r * math.cos(phi), r * math.sin(phi), -0.25
    q = O.qdeposit(g, pl)
    k = 4                       # cell index: nodes k+1 (r = k dr) and k+2
    assert q[0, 0, k + 1] == pytest.approx(-0.25 * (1 - f) / k)
    assert q[0, 0, k + 2] == pytest.approx(-0.25 * f / (k + 1))
    assert q[1, 0, k + 1] == pytest.approx(-0.25 * (1 - f) * math.cos(phi) / k)       # Re e^{-i phi}
    assert q[2, 0, k + 1] == pytest.approx(-0.25 * (1 - f) * -math.sin(phi) / k)      # Im e^{-i phi}
    assert q[3, 0, k + 2] == pytest.approx(-0.25 * f * math.cos(2 * phi) / (k + 1))
    assert np.count_nonzero(q) == 2 * 5


def test_single_particle_axis_rules():
    """A particle in the first cell: m=0 node 1 is multiplied by 8, m>0 node 1 is zero."""
    g = O.grid(8, 1, 1, 0.1, 0.1)
    pl = O.Plasma(1)
    pl.x[0], pl.y[0], pl.q[0] = 0.04, 0.0, 1.0
    q = O.qdeposit(g, pl)
    assert q[0, 0, 1] == pytest.approx(8 * 0.6) and q[0, 0, 2] == pytest.approx(0.4)
    assert q[1, 0, 1] == 0.0 and q[1, 0, 2] == pytest.approx(0.4)


def test_push_in_uniform_ez():
    """Robust push of a particle at rest in a uniform Ez: pz = qbm Ez dt, x unchanged in r."""
    nr, dr, dt, ez = 16, 0.1, 0.05, 0.7
    g = O.grid(nr, 1, 1, dr, dt)
    ef, bf = O.field(g, 3), O.field(g, 3)
    ef[0, 2, :] = ez
    pl = O.Plasma(1)
    pl.x[0], pl.y[0], pl.q[0], pl.gamma[0] = 0.35, 0.2, -1.0, 1.0
    O.push_u(g, O.PUSH_ROBUST, -1.0, dt, pl, ef, bf)
    assert pl.pz[0] == pytest.approx(-1.0 * ez * dt, rel=1e-14)
    assert pl.px[0] == 0.0 and pl.py[0] == 0.0
    assert pl.gamma[0] == pytest.approx(math.sqrt(1 + (ez * dt) ** 2))


def test_push_in_uniform_bz_rotates():
    nr, dr, dt = 16, 0.1, 0.05
    g = O.grid(nr, 1, 1, dr, dt)
    ef, bf = O.field(g, 3), O.field(g, 3)
    bf[0, 2, :] = 2.0
    pl = O.Plasma(1)
    pl.x[0], pl.y[0], pl.px[0], pl.py[0], pl.q[0] = 0.35, 0.2, 0.3, -0.1, -1.0
    pl.gamma[0] = math.sqrt(1 + 0.1)
    O.push_u(g, O.PUSH_ROBUST, -1.0, dt, pl, ef, bf)
    assert math.hypot(pl.px[0], pl.py[0]) == pytest.approx(math.hypot(0.3, 0.1), rel=1e-14)
    assert pl.pz[0] == 0.0


def test_update_bound_swaps_last_particle_in():
    g = O.grid(10, 1, 0, 0.1, 0.1)                   # edge = 1.0
    pl = O.Plasma(5)
    pl.x[:] = [0.5, 1.1, 0.3, 1.2, 0.1]
    pl.q[:] = [1, 2, 3, 4, 5]
    n = O.update_bound(g, pl)
    assert n == 3
    assert list(pl.q[:3]) == [1, 5, 3]
    assert list(pl.x[:3]) == [0.5, 0.1, 0.3]


def test_counting_sort_permutation():
    """generate_sort_idx_1d: the first particle of a cell goes to the cell's last slot."""
    g = O.grid(3, 1, 0, 1.0, 0.1)
    pl = O.Plasma(5)
    pl.x[:] = [1.5, 0.5, 1.2, 2.5, 0.7]              # keys 2, 1, 2, 3, 1
    pl.q[:] = [1, 2, 3, 4, 5]
    keys, idx = O.sort(g, pl)
    assert list(keys) == [2, 1, 2, 3, 1]
    assert list(idx) == [4, 2, 3, 5, 1]
    assert list(pl.q) == [5, 2, 3, 1, 4]


def test_neutral_plasma_without_driver_stays_at_rest():
    """No beam: rho - Jz cancels the neutralising background exactly; every field stays 0.
    The convergence test then never passes (old norm 0 -> rel_res = huge) and the loop
    runs to iter_max, as simulation_class.f03:394-396 does."""
    g = O.grid(32, 6, 1, 0.1, 0.1)
    pl = O.load_plasma(g, 1, 2, 1, 8)
    sim = O.Sim(g, iter_max=3, sp_npmax=pl.n)
    sim.set_plasma(pl)
    iters, rel = sim.run_3dstep(push_beams=False)
    assert list(iters) == [3] * 6
    assert np.all(rel > 1e300)
    for name in ("psi", "e", "b", "cu"):
        assert np.count_nonzero(sim.store(name)) == 0, name
    out = sim.plasma()
    assert out.n == pl.n and np.array_equal(out.x, pl.x)


def test_linear_wake_period():
    """Weak driver (n_b = 0.01): on-axis Ez behind the beam oscillates at k_p = 1."""
    nr, nz, dr, dxi = 96, 448, 0.05, 0.05
    g = O.grid(nr, nz, 0, dr, dxi)
    pl = O.load_plasma(g, 0, 2, 1, 8)
    sr, sz, nb = 0.5, 0.5, 0.01
    Q = nb * (2 * math.pi) ** 1.5 * sr * sr * sz
    bm = O.load_beam(g, 3, 100000, Q, -1.0, 20000.0, (0, 0, 2.0), (sr, sr, sz), (-2.5, -2.5, 0.0), (2.5, 2.5, 4.5))
    sim = O.Sim(g, iter_max=40, sp_npmax=pl.n, beams=[(-1.0, O.PUSH3_REDUCED, bm.n)], nthreads=4)
    sim.set_plasma(pl)
    sim.set_beam(0, bm)
    sim.run_3dstep(push_beams=False)
    ez = sim.store("e")[:nz, 0, 2, 1]
    xi = np.arange(nz) * dxi
    tail = xi > 5.0
    zc = xi[tail][np.where(np.diff(np.sign(ez[tail])) != 0)[0]]
    period = 2 * float(np.mean(np.diff(zc)))
    assert abs(period - 2 * math.pi) / (2 * math.pi) < 0.03, period
    assert ez[(xi > 1.0) & (xi < 2.5)].max() > 0            # decelerating field inside an electron driver


def test_smooth_known_answer():
    """One binomial smoothing pass (ufield_class.f03:274-339) written out by hand: kernel
    (1, 2, 1)/4; node 1 the axis form where the mode/component switch is set (else 0), node 2
    the near-axis form, nodes j >= 3 weighted by (1 -+ 1/(j-1)); guards unchanged.  Switches:
    rho m=0; jay m=0 comp 2 and m=1 comps 0, 1; djdxi m=1 (field_src_class.f03)."""
    nr, M = 7, 2
    g = O.grid(nr, 4, M, 0.1, 0.1)
    P, ld = 2 * M + 1, nr + 2
    rng = np.random.default_rng(12)
    for kind, nc in ((0, 1), (1, 3), (2, 2)):
        f = rng.standard_normal(P * nc * ld)
        got = O.smooth(g, kind, f.copy()).reshape(P, nc, ld)
        v = f.reshape(P, nc, ld)
        for p in range(P):
            m = (p + 1) // 2
            for c in range(nc):
                ax = {0: m == 0, 1: (c == 2) if m == 0 else (m == 1 and c < 2), 2: m == 1}[kind]
                w = v[p, c]
                exp = w.copy()
                exp[1] = (0.5 + 0.25) * w[1] + 8.0 * 0.25 * w[2] if ax else 0.0
                exp[2] = 0.5 * w[2] + 0.125 * 0.25 * w[1] + 2.0 * 0.25 * w[3]
                for j in range(3, nr + 1):
                    r = float(j - 1)
                    exp[j] = 0.5 * w[j] + (1.0 - 1.0 / r) * 0.25 * w[j - 1] + (1.0 + 1.0 / r) * 0.25 * w[j + 1]
                assert np.array_equal(got[p, c], exp), (kind, p, c)
    # a constant is preserved away from the axis
    f = np.ones(P * ld)
    O.smooth(g, 0, f)
    assert np.all(f.reshape(P, ld)[:, 3:nr + 1] == 1.0)


def test_two_beams_deposit_as_their_sum():
    """beam3d::qdp (beam3d_class.f03:193-221): every beam deposits into its own zeroed store,
    finished by part3d::qdeposit (axis rule, 1/(i-1)), then added to q_beam; two beams give
    the same store as one beam holding both beams' particles."""
    g = O.grid(32, 16, 2, 0.1, 0.1)
    b1 = O.load_beam(g, 5, 4000, 3.0, -1.0, 1000.0, (0.05, 0.0, 0.6), (0.3, 0.3, 0.2), (-1.5, -1.5, 0.0),
                     (1.5, 1.5, 1.6))
    b2 = O.load_beam(g, 6, 3000, 2.0, -1.0, 1000.0, (0.0, 0.0, 1.0), (0.2, 0.2, 0.2), (-1.0, -1.0, 0.0),
                     (1.0, 1.0, 1.6))
    both = O.Beam(b1.n + b2.n)
    for k in O.Beam.NAMES:
        setattr(both, k, np.ascontiguousarray(np.concatenate([getattr(b1, k), getattr(b2, k)])))
    stores = []
    for beams in ([b1, b2], [both]):
        sim = O.Sim(g, iter_max=1, sp_npmax=1, beams=[(-1.0, O.PUSH3_REDUCED, b.n) for b in beams])
        for k, b in enumerate(beams):
            sim.set_beam(k, b)
        sim.begin_3dstep()
        stores.append(sim.store("q_beam"))
    sep = O.beam_qdeposit(g, b1) + O.beam_qdeposit(g, b2)
    np.testing.assert_allclose(stores[0], stores[1], rtol=0, atol=1e-12 * np.abs(stores[1]).max())
    np.testing.assert_allclose(stores[0][:g.nz], sep[:g.nz], rtol=0, atol=1e-12 * np.abs(sep).max())
