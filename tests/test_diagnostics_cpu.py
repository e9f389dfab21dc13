"""Host-side diagnostics and helpers: the per-mode error report of the benchmark and the choice
of trained weights (no GPU)."""
import os

import numpy as np

from qpad_gb300 import learned as LR
from qpad_gb300.diagnostics import mode_errors, step_error_report


def _store(nz=6, M=2, ncomp=3, nr=10, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nz, 2 * M + 1, ncomp, nr + 2))


def test_mode_errors_per_mode_and_against_the_field():
    ref = _store()
    ref[:, 1:] *= 1e-3                            # modes m >= 1 small next to m = 0
    got = ref.copy()
    got[:, 3, 1, 4] += 1e-4                       # an error in the Re part of m = 2, component 1
    got[2, 0, 0, 2] += 5e-3                       # an error in m = 0, component 0, slice 3
    err = mode_errors(got, ref, 2)
    r2 = ref[:, [3, 4], 1, 1:]
    d2 = got[:, [3, 4], 1, 1:] - r2
    want = np.linalg.norm(d2) / np.linalg.norm(r2)
    assert abs(err[(2, 1)][0] - want) <= 1e-12 * want
    assert abs(err[(2, 1)][3] - np.linalg.norm(d2) / np.linalg.norm(ref[:, :, 1, 1:])) <= 1e-12 * want
    assert err[(2, 1)][3] < err[(2, 1)][0]       # relative to the whole field it is smaller
    assert err[(0, 0)][1] == 3                    # the worst slice (1-based)
    assert err[(1, 2)][0] == 0.0


def test_mode_errors_skip_modes_below_the_floor():
    ref = _store(M=1)
    ref[:, 1:] = 1e-12 * ref[:, 1:]               # m = 1 holds round-off only
    err = mode_errors(ref + 1e-14, ref, 1)
    assert all(m == 0 for (m, _) in err)


def test_step_error_report_names_the_worst():
    ref = {"psi": _store(ncomp=1, seed=1), "e": _store(seed=2)}
    got = {k: v.copy() for k, v in ref.items()}
    got["e"][:, 2, 2, :] *= 1.01                  # Im of m = 1, E_z: 1 % of that part
    rep = step_error_report(got, ref, 2)
    assert rep["worst"] == "e[2] m=1"
    assert 0.0 < rep["max_vs_field"] < rep["max"]
    assert rep["worst_vs_field"] == "e[2] m=1"
    assert set(rep["per_mode"]) == set(rep["per_mode_vs_field"])
    empty = step_error_report({}, {}, 2)
    assert empty["max"] is None and empty["max_vs_field"] is None


def test_weights_path_serves_every_mode_count():
    c2 = os.path.join(LR.WEIGHTS, "guess_c2.npz")
    for M in (0, 1, 2):
        assert LR.weights_path(M) == c2
    c5 = os.path.join(LR.WEIGHTS, "guess_c5.npz")
    assert LR.weights_path(4) == (c5 if os.path.exists(c5) else c2)
