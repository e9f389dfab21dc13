"""qpad_species_amjdp_noalloc: the current deposit that allocates no device memory.

Called through the C ABI and checked against qpad_species_amjdp on the same particles and
fields, on two calls in a row (the static scratch keeps the first call's contents, so the
second call shows that it is cleared).  Tolerances are those of the deposit parity tests:
1e-10 relative L2 for FP64 (atomic summation order), 5e-5 for the mixed path.
"""
import ctypes as C

import numpy as np
import pytest

import qpad_gb300 as Q
from oracle import oracle as O
from qpad_gb300 import _capi as K
from tests.helpers import field_errors, smooth_field

pytestmark = pytest.mark.gpu

TOL = {K.PREC_FP64: 1e-10, K.PREC_MIXED: 5e-5}


def _plasma(nr, dr, seed, uth=0.05):
    x, p, g, ps, q = Q.load_plasma(nr, dr, seed, 2, 2, 8, uth=(uth, uth, uth))
    rng = np.random.default_rng(seed)
    x = np.ascontiguousarray(x + rng.uniform(-0.45, 0.45, x.shape) * dr)
    ps = np.ascontiguousarray(rng.uniform(-0.2, 0.2, len(q)))
    return x, p, g, ps, q


def _deposit(sim, sp, fn, dt):
    for f in (sim.cu, sim.amu, sim.acu):
        f.fill(0.0)
    r = fn(sp.h, sim.e.id, sim.b.id, sim.cu.id, sim.amu.id, sim.acu.id, C.c_double(dt))
    assert r == K.OK, sim.lib.qpad_last_error(sim.h).decode()
    return [f.download() for f in (sim.cu, sim.amu, sim.acu)]


@pytest.mark.parametrize("precision", [K.PREC_FP64, K.PREC_MIXED])
@pytest.mark.parametrize("push_type", [O.PUSH_ROBUST, O.PUSH_STD])
def test_noalloc_matches_amjdp(precision, push_type):
    nr, M, dr, dt = 128, 2, 0.04, 0.04
    g = O.grid(nr, 4, M, dr, dt)
    rng = np.random.default_rng(300 + precision + push_type)
    sim = Q.Simulation(nr, 4, M, dr, dt, precision=precision)
    sim.e.upload(smooth_field(rng, g, 3, scale=0.5))
    sim.b.upload(smooth_field(rng, g, 3, scale=0.5))
    x, p, gam, ps, q = _plasma(nr, dr, 31 + precision)
    sp = sim.add_species(x, p, gam, ps, q, push_type=push_type)
    ref = _deposit(sim, sp, sim.lib.qpad_species_amjdp, dt)
    assert max(np.abs(a).max() for a in ref) > 0
    for call in range(2):
        got = _deposit(sim, sp, sim.lib.qpad_species_amjdp_noalloc, dt)
        for name, a, b in zip(("cu", "amu", "dcu"), got, ref):
            err = field_errors(a, b, nodes=slice(0, None)).max()
            assert err < TOL[precision], (call, name, err)
    sim.close()


def test_noalloc_rejects_grid_beyond_limit():
    # 8 * (2*4+1) * (2000+2) doubles > 131072: refused before anything is launched
    sim = Q.Simulation(2000, 4, 4, 0.01, 0.04)
    x, p, gam, ps, q = _plasma(64, 0.01, 7)
    sp = sim.add_species(x, p, gam, ps, q)
    r = sim.lib.qpad_species_amjdp_noalloc(sp.h, sim.e.id, sim.b.id, sim.cu.id, sim.amu.id, sim.acu.id,
                                           C.c_double(0.04))
    assert r == K.E_CAPACITY
    assert b"limit" in sim.lib.qpad_last_error(sim.h)
    sim.close()
