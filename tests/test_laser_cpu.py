"""Laser envelope on the CPU: the oracle's restatement of the reference's penta-diagonal
cyclic reduction (fpcr_penta_class.f03) against dense solves, the envelope advance
(field_laser_class.f03) against the diffraction of a Gaussian beam in vacuum, and the
susceptibility deposit (part2d_class.f03:361-476) against the charge deposit."""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from qpad_gb300 import lasers as LZ

EPS = 2.220446049250313e-16


def _dense(A):
    n = A.shape[1]
    Md = np.zeros((n, n))
    for i in range(n):
        for k, off in enumerate((-2, -1, 0, 1, 2)):
            if 0 <= i + off < n:
                Md[i, i + off] = A[k, i]
    return Md


def test_pcr_solves_a_penta_diagonal_system():
    rng = np.random.default_rng(2)
    n = 128
    A = rng.normal(size=(5, n))
    A[2] = 6.0 + rng.random(n)
    # out-of-range couplings as the reference sets them (set_values_matrix_byrow)
    A[0, 0] = A[1, 0] = A[0, 1] = EPS
    A[4, -2] = A[3, -1] = A[4, -1] = EPS
    rhs = rng.normal(size=n)
    x = O.pcr_solve(O.pcr_coef(A), rhs)
    xd = np.linalg.solve(_dense(A), rhs)
    assert np.abs(x - xd).max() <= 1e-13 * np.abs(xd).max()


@pytest.mark.parametrize("m", [0, 1, 2, 3])
def test_pcr_solves_the_envelope_system(m):
    nr = 64
    A = O.laser_matrix(nr, m, 10.0, 1.0, 0.05, 0.1)
    rng = np.random.default_rng(m)
    rhs = rng.normal(size=2 * nr)
    if m > 0:
        rhs[:2] = 0.0        # the axis rows of m >= 1 carry no source in the loop
    x = O.pcr_solve(O.pcr_coef(A), rhs)
    xd = np.linalg.solve(_dense(A), rhs)
    assert np.abs(x - xd).max() <= 1e-12 * np.abs(xd).max()


def test_gaussian_beam_diffracts_in_vacuum():
    """No plasma: the envelope of a long pulse obeys the paraxial equation, so the on-axis
    amplitude of a Gaussian beam launched at its waist falls as w0 / w(s),
    w(s) = w0 sqrt(1 + (s / z_R)^2), z_R = k0 w0^2 / 2."""
    nr, nz, dr, dxi = 64, 64, 0.05, 0.1
    k0, w0, a0, ds, nsteps = 10.0, 1.0, 0.1, 0.5, 10
    g = O.grid(nr, nz, 1, dr, dxi)
    # a pulse at its waist in every slice (flat phase), sin^2 envelope along xi
    P = 3
    ar, ai = np.zeros((nz, P, nr)), np.zeros((nz, P, nr))
    r = np.arange(nr) * dr
    for j in range(nz):
        ar[j, 0] = a0 * LZ.longitudinal(j * dxi - 3.2, ("sin2", 2.0, 1.0, 2.0)) * np.exp(-r * r / (w0 * w0))
    sim = O.Sim(g, iter_max=5, dt3d=ds, sp_npmax=1, sp_push_type=O.PUSH_ROBUST_PGC,
                lasers=[dict(k0=k0, iter=1, ar=ar, ai=ai)])
    sim.set_plasma(O.Plasma(0))
    jc = int(round(3.2 / dxi))               # the pulse centre's slice
    zr = 0.5 * k0 * w0 * w0
    for step in range(1, nsteps + 1):
        sim.run_3dstep(push_beams=False)
        lr, li = sim.laser(0)
        amp = np.hypot(lr[jc - 1, 0, 1], li[jc - 1, 0, 1])
        want = a0 / np.sqrt(1.0 + (step * ds / zr) ** 2)
        assert abs(amp / want - 1.0) < 0.01, (step, amp, want)


def test_chi_deposit_is_the_scaled_charge_deposit():
    """Cold plasma (psi = 0): chi = -qbm * (charge deposit) off the axis; on the axis the
    charge deposit's factor 8 is replaced by 12 ppc_r^2 / (1 + 2 ppc_r^2)."""
    nr, M = 32, 2
    g = O.grid(nr, 4, M, 0.1, 0.1)
    rng = np.random.default_rng(7)
    n = 4000
    r = np.sqrt(rng.random(n)) * nr * 0.1 * 0.999
    th = rng.random(n) * 2 * np.pi
    x, y = r * np.cos(th), r * np.sin(th)
    q = -rng.random(n)
    psi = np.zeros(n)
    P = 2 * M + 1
    chi = np.zeros((P, nr + 2))
    qd = np.zeros((P, nr + 2))
    qbm, ppc_r = -1.0, 3
    O.lib().orc_deposit_chi(ctypes.byref(g), qbm, ppc_r, n, O.ptr(x), O.ptr(y), O.ptr(q), O.ptr(psi), O.ptr(chi))
    O.lib().orc_qdeposit(ctypes.byref(g), n, O.ptr(x), O.ptr(y), O.ptr(q), O.ptr(qd))
    corr = 12.0 * ppc_r ** 2 / (1.0 + 2.0 * ppc_r ** 2)
    np.testing.assert_allclose(chi[:, 2:], -qbm * qd[:, 2:], rtol=1e-12, atol=1e-14)
    assert np.isclose(chi[0, 1], -qbm * qd[0, 1] / 8.0 * corr, rtol=1e-12)
    assert np.all(chi[1:, 1] == 0.0) and np.all(chi[:, 0] == 0.0)
