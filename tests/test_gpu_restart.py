"""Restart and diagnostic files through the device.

* Beams saved after a 3D step (the reference's HDF5 restart files) come back on a new context
  with the same particles, and one more 3D step from the restored state equals one more 3D step
  of the original (iteration counts and fields).
* The field dumps of a 3D step (the reference's per-mode HDF5 files) hold the device's 3D
  stores, checked with an independent parser of the format.
"""
import os

import numpy as np
import pytest

import qpad_gb300 as Q
from qpad_gb300 import restart
from qpad_gb300.diagnostics import FIELD_DIAGS, mode_dirs, write_field_diags
from tests import h5_parse

pytestmark = pytest.mark.gpu


def _deck():
    return Q.decks.Deck("rst", nr=48, nz=16, max_mode=1, dr=0.05, dxi=0.05, ppc=(2, 1), num_theta=8,
                        uth=1e-3, seed=4, beams=[Q.decks.BeamSpec(2.0, 0.4, 0.3, 0.4, 3000, x0=0.02),
                                                 Q.decks.BeamSpec(1.0, 0.3, 0.2, 0.6, 2000)],
                        iter_max=20, iter_reltol=1e-6)


def test_beam_restart_round_trip_and_next_step(tmp_path):
    deck = _deck()
    pl, beams = Q.deck_inputs(deck)
    a = Q.build_simulation(deck, inputs=(pl, beams))
    a.run_3d_step()
    restart.save_beams(a, str(tmp_path), timestep=1)
    b = Q.Simulation(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi, iter_max=deck.iter_max,
                     iter_reltol=deck.iter_reltol, dt=deck.dt)
    b.add_species(*pl)
    restart.load_beams(b, str(tmp_path), timestep=1, nbeams=2)
    for ba, bb in zip(a.beams, b.beams):
        for u, v in zip(ba.download(), bb.download()):
            assert np.array_equal(u, v)
    # the next 3D step from the restored beams equals the original's next step
    a.species[0].reset()
    ia, _ = a.run_3d_step()
    ib, _ = b.run_3d_step()
    assert np.array_equal(ia, ib)
    for name in ("e", "b", "psi"):
        d = np.abs(a.fields[name].store_all() - b.fields[name].store_all()).max()
        assert d <= 1e-12 * np.abs(a.fields[name].store_all()).max(), name
    # (the FP64 deposits add with atomics in no fixed order: the pushed beams agree to round-off)
    for ba, bb in zip(a.beams, b.beams):
        for u, v in zip(ba.download(), bb.download()):
            np.testing.assert_allclose(u, v, rtol=1e-12, atol=1e-14)
    a.close()
    b.close()


def test_field_dumps_hold_the_stores(tmp_path):
    deck = _deck()
    sim = Q.build_simulation(deck)
    sim.run_3d_step()
    names = ["ez_cyl_m", "bphi_cyl_m", "psi_cyl_m", "charge_cyl_m"]
    write_field_diags(sim, names, str(tmp_path), tstep=3)
    for n in names:
        field, comp, sub, dataname, units, label = FIELD_DIAGS[n]
        store = sim.fields[field].store_all()
        for part, d in enumerate(mode_dirs(deck.max_mode)):
            path = os.path.join(str(tmp_path), "Fields", sub, d, f"{dataname}_00000003.h5")
            f = h5_parse.File(path)
            assert f.members() == ["AXIS", dataname]
            assert np.array_equal(f.dataset(dataname), store[:, part, comp, 1:deck.nr + 1])
            assert f.attrs["ITER"] == [3] and f.attrs["TIME"] == [3 * deck.dt]
            assert f.obj(dataname)["attrs"]["LONG_NAME"].rstrip() == label
            assert f.dataset("AXIS/AXIS1").tolist() == [0.0, deck.nr * deck.dr]
    sim.close()
