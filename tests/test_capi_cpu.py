"""CPU-side checks of the product library: it loads without a GPU, exports every symbol
the header declares, and its host loaders match the oracle's bit for bit."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT


def _declared():
    txt = open(os.path.join(ROOT, "include", "qpad_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(qpad_[a-z0-9_]+)\s*\(", txt)))


def test_header_symbols_exported(qlib):
    names = _declared()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(qlib, n)]
    assert not missing, missing


def test_python_bindings_cover_header():
    from qpad_gb300 import _capi
    assert sorted(_capi.EXPORTED) == _declared()


def test_device_count_without_gpu_is_clean(qlib):
    n = C.c_int(-1)
    assert qlib.qpad_device_count(C.byref(n)) == 0
    assert n.value >= 0


def test_create_rejects_bad_grid(qlib):
    from qpad_gb300 import _capi as K
    d = K.GridDesc(4, 10, 1, K.BND_OPEN, 0.1, 0.1, -1.0, 10, 1e-6, 0.0, 1.0, 0, 0)   # nr < 8
    h = C.c_void_p()
    assert qlib.qpad_ctx_create(C.byref(d), C.byref(h)) == K.E_ARG
    assert b"invalid grid" in qlib.qpad_last_error(None)
    d = K.GridDesc(64, 10, 9, K.BND_OPEN, 0.1, 0.1, -1.0, 10, 1e-6, 0.0, 1.0, 0, 0)   # max_mode > 8
    assert qlib.qpad_ctx_create(C.byref(d), C.byref(h)) == K.E_ARG


def test_plasma_loader_matches_oracle(olib):
    import qpad_gb300 as Q
    g = olib.grid(96, 8, 1, 0.03, 0.03)
    ref = olib.load_plasma(g, 5, 4, 2, 8, uth=(1e-3, 2e-3, 3e-3))
    x, p, gam, ps, q = Q.load_plasma(96, 0.03, 5, 4, 2, 8, uth=(1e-3, 2e-3, 3e-3))
    assert len(q) == ref.n == 96 * 4 * 2 * 8
    for a, b in ((x[:, 0], ref.x), (x[:, 1], ref.y), (p[:, 0], ref.px), (p[:, 1], ref.py), (p[:, 2], ref.pz),
                 (gam, ref.gamma), (ps, ref.psi), (q, ref.q)):
        np.testing.assert_array_equal(a, b)


def test_beam_loader_matches_oracle(olib):
    import qpad_gb300 as Q
    nr, nz, dr, dxi = 128, 64, 0.04, 0.04
    g = olib.grid(nr, nz, 1, dr, dxi)
    spec = Q.decks.BeamSpec(3.0, 0.5, 0.6, 1.8, 20000, x0=0.05)
    a = spec.load_args(nz, dxi)
    x, p, q = Q.load_beam(nr, nz, dr, dxi, 9, **a)
    ref = olib.load_beam(g, 9, a["tot_num"], a["tot_charge"], a["qm"], a["gamma"], a["center"], a["sigma"],
                         a["range_lo"], a["range_hi"], a["uth"])
    assert len(q) == ref.n
    for u, v in ((x[:, 0], ref.x), (x[:, 1], ref.y), (x[:, 2], ref.z), (p[:, 0], ref.px), (p[:, 2], ref.pz),
                 (q, ref.q)):
        np.testing.assert_array_equal(u, v)
    # quiet start mirrors every particle and halves the charge (fdist3d_rnd_class.f03:459-489)
    xq, pq, qq = Q.load_beam(nr, nz, dr, dxi, 9, quiet=True, **a)
    n = len(q)
    assert len(qq) == 2 * n
    np.testing.assert_array_equal(xq[n:, :2], -xq[:n, :2])
    np.testing.assert_array_equal(qq[:n], 0.5 * q)


def test_beam_loader_rejects_empty_range():
    """An empty sampling range is an error, not an endless rejection loop."""
    import qpad_gb300 as Q
    with pytest.raises(Q.QpadError):
        Q.load_beam(32, 16, 0.1, 0.1, 5, 100, 1.0, -1.0, 1000.0, (0.0, 0.0, 3.0), (0.1, 0.1, 0.2),
                    (-0.5, -0.5, 3.0), (0.5, 0.5, 1.6))


def test_deck_inputs_skip_beam_behind_short_box():
    import qpad_gb300 as Q
    deck = Q.decks.c2().scaled(nz=48)
    pl, beams = Q.deck_inputs(deck)
    assert len(beams) == 2 and len(beams[1][2]) == 0 and len(beams[0][2]) > 0


def _prototypes():
    """{name: argument count} of every function the header declares."""
    txt = open(os.path.join(ROOT, "include", "qpad_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    out = {}
    for m in re.finditer(r"\b(qpad_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_python_bindings_match_header_arity():
    """Every ctypes declaration takes as many arguments as the header's prototype."""
    from qpad_gb300 import _capi
    protos = _prototypes()
    assert set(protos) == set(_capi.EXPORTED)
    bad = {n: (protos[n], len(_capi._SIGS[n][1])) for n in protos if protos[n] != len(_capi._SIGS[n][1])}
    assert not bad, bad
