"""The reference's JSON input deck (json-fortran dialect) read into this library's setup:
keys, derived grid quantities, the accepted subset and refusals, and the particle inputs the
CPU loaders make from it."""
import copy
import json
import os

import numpy as np
import pytest

from qpad_gb300 import _capi as K
from qpad_gb300 import inputdeck as ID

DECK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "decks", "two_beams.json")


def _raw():
    with open(DECK) as f:
        return json.loads(ID.strip_comments(f.read()))


def test_comments_stripped_outside_strings():
    assert ID.strip_comments('{"a" : 1 ! note\n}') == '{"a" : 1 \n}'
    assert json.loads(ID.strip_comments('{"a" : "x!y" ! c\n}')) == {"a": "x!y"}


def test_parse_simulation_species_beams():
    d = ID.read(DECK)
    assert (d.nr, d.nz, d.max_mode) == (128, 96, 2)
    assert d.dr == pytest.approx(0.04) and d.dxi == pytest.approx(0.04)
    assert d.n_steps == 3 and d.dt == 10.0 and d.seed == 7
    assert (d.iter_max, d.iter_reltol, d.iter_abstol) == (40, 1e-5, 1e-12)
    assert d.bnd == K.BND_OPEN and d.relax_fac is None and d.start_step == 1
    (s,) = d.species
    assert s["ppc"] == (2, 2) and s["num_theta"] == 8 and s["push_type"] == K.PUSH2_STD
    assert s["neutralized"] and s["smooth_order"] == 1 and s["qbm"] == -1.0
    b1, b2 = d.beams
    assert b1["tot_num"] == 20000 and b1["tot_charge"] == 3.5 and b1["push_type"] == K.PUSH3_REDUCED
    assert b1["center"] == (0.03, 0.0, 1.2) and b1["range_hi"] == (1.5, 1.5, 3.2)
    assert b2["qbm"] == -0.5 and b2["push_type"] == K.PUSH3_BORIS and b2["uth"] == (0.0, 0.0, 0.0)


def test_restart_start_step():
    raw = _raw()
    raw["simulation"]["read_restart"] = True
    assert ID.parse(raw).start_step == 5      # restart_timestep + 1 (simulation_class.f03:150-155)


@pytest.mark.parametrize("path,value", [
    (("simulation", "nlasers"), 1),
    (("simulation", "nneutrals"), 2),
    (("simulation", "interpolation"), "quadratic"),
    (("beam", 0, "profile_type"), "standard"),
    (("beam", 1, "profile"), ["gaussian", "gaussian", "uniform"]),
    (("species", 0, "profile"), ["uniform", "piecewise-linear"]),
    (("simulation", "box", "z"), [1.0, 4.84]),
    (("simulation", "algorithm"), "subcycling"),
    (("beam", 0, "alpha"), [0.5, 0.5]),
    (("beam", 0, "perp_offset_x"), [0.0, 0.1]),
    (("beam", 1, "perp_offset_y"), [0.0, 0.1]),
    (("beam", 1, "has_spin"), True),
])
def test_unsupported_features_refused(path, value):
    raw = copy.deepcopy(_raw())
    node = raw
    for k in path[:-1]:
        node = node[k]
    node[path[-1]] = value
    with pytest.raises(NotImplementedError):
        ID.parse(raw)


def test_missing_required_key():
    raw = _raw()
    del raw["simulation"]["iter_max"]
    with pytest.raises(ValueError):
        ID.parse(raw)


def test_inputs_from_the_loaders():
    d = ID.read(DECK)
    (pl,), (b1, b2) = ID.inputs(d)
    x, p, g, ps, q = pl
    assert len(q) == d.nr * 2 * 2 * 8 and x.shape == (len(q), 2)
    for (bx, bp, bq), spec in zip((b1, b2), d.beams):
        assert len(bq) == spec["tot_num"] and bx.shape == (len(bq), 3)
        lo, hi = np.array(spec["range_lo"]), np.array(spec["range_hi"])
        assert np.all(bx >= lo - 1e-12) and np.all(bx <= hi + 1e-12)
    # the same seed gives the same particles
    (pl2,), _ = ID.inputs(d)
    assert np.array_equal(pl2[0], x)


def test_run_renews_plasma_before_later_steps():
    d = ID.read(DECK)

    class _Sp:
        def __init__(self):
            self.renewed = []

        def renew(self, x, p, g, ps, q):
            self.renewed.append(x.copy())

    class _Sim:
        def __init__(self):
            self.species, self.steps = [_Sp()], 0

        def run_3d_step(self):
            self.steps += 1
            return np.zeros(d.nz, np.int32), np.zeros(d.nz)

    sim = _Sim()
    out = ID.run(d, sim)
    assert sim.steps == d.n_steps == len(out)
    assert len(sim.species[0].renewed) == d.n_steps - 1
    (pl2,), _ = ID.inputs(d, d.start_step + 1)
    assert np.array_equal(sim.species[0].renewed[0], pl2[0])


def _counting_sim(d):
    class _Sp:
        def renew(self, *a):
            pass

    class _Sim:
        def __init__(self):
            self.species, self.steps = [_Sp() for _ in d.species], 0

        def run_3d_step(self):
            self.steps += 1
            return np.zeros(d.nz, np.int32), np.zeros(d.nz)
    return _Sim()


def test_restart_runs_only_the_remaining_steps():
    # the reference loops i = start3d .. nstep3d (simulation_class.f03:294)
    raw = _raw()
    raw["simulation"]["read_restart"] = True
    d = ID.parse(raw)
    for rst, expect in ((0, d.n_steps), (1, d.n_steps - 1), (d.n_steps - 1, 1), (d.n_steps, 0), (d.n_steps + 3, 0)):
        raw["simulation"]["restart_timestep"] = rst
        dd = ID.parse(raw)
        assert dd.start_step == rst + 1
        sim = _counting_sim(dd)
        assert len(ID.run(dd, sim)) == expect == sim.steps


def test_loader_streams_distinct():
    seeds = {ID.stream_seed(7, 0, k, s) for k in range(3) for s in range(1, 1200)}
    seeds |= {ID.stream_seed(7, 1, k) for k in range(4)}
    assert len(seeds) == 3 * 1199 + 4
    assert ID.stream_seed(7, 0, 1, 5) == ID.stream_seed(7, 0, 1, 5)
