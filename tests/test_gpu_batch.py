"""Batched simulations (one graph launch for the slice loops of all of them) and the
autotuner, against the same simulations run one by one."""
import numpy as np
import pytest

import qpad_gb300 as Q
from tests.helpers import store_errors

pytestmark = pytest.mark.gpu


def _decks():
    out = []
    for k, (nr, M) in enumerate([(64, 0), (96, 2), (48, 1)]):
        out.append(Q.decks.Deck(f"batch_{k}", nr=nr, nz=32, max_mode=M, dr=0.04, dxi=0.04, ppc=(2, 1),
                                num_theta=8, uth=2e-3, seed=11 + k,
                                beams=[Q.decks.BeamSpec(1.5 + k, 0.4, 0.3, 0.5, 10000, x0=0.03)],
                                iter_max=30, iter_reltol=1e-6))
    return out


@pytest.mark.parametrize("precision", [Q._capi.PREC_FP64, Q._capi.PREC_MIXED])
def test_batch_step_matches_single_steps(precision):
    decks = _decks()
    single = [Q.build_simulation(d, precision=precision) for d in decks]
    its_single = [s.run_3d_step()[0] for s in single]
    sims = [Q.build_simulation(d, precision=precision) for d in decks]
    batch = Q.Batch(sims)
    its_batch = batch.step()
    tol = 1e-9 if precision == Q._capi.PREC_FP64 else 1e-4
    for d, a, b, ia, ib in zip(decks, single, sims, its_single, its_batch):
        if precision == Q._capi.PREC_FP64:
            assert np.array_equal(ia, ib), (d.name, ia, ib)
        else:
            assert abs(float(ia.mean()) - float(ib.mean())) < 0.5
        for f in ("e", "b", "psi"):
            ga = np.stack([a.fields[f].store(s) for s in range(1, d.nz + 1)])
            gb = np.stack([b.fields[f].store(s) for s in range(1, d.nz + 1)])
            assert store_errors(gb, ga).max() < tol, (d.name, f)
    # a second step reuses the batch graph
    its2 = batch.step()
    assert all(len(i) == d.nz for i, d in zip(its2, decks))
    batch.close()
    for s in single + sims:
        s.close()


@pytest.mark.parametrize("precision", [Q._capi.PREC_FP64, Q._capi.PREC_MIXED])
def test_autotune_keeps_results(precision):
    d = _decks()[1]
    a = Q.build_simulation(d, precision=precision)
    ia, _ = a.run_3d_step()
    b = Q.build_simulation(d, precision=precision)
    res = b.autotune(reps=5)
    assert res["iter_cluster"] in (1, 2, 4, 8, 16) and res["iter_us"] > 0
    assert res["item_ppl"] in (1, 2, 4)
    ib, _ = b.run_3d_step()
    tol = 1e-9 if precision == Q._capi.PREC_FP64 else 1e-4
    if precision == Q._capi.PREC_FP64:
        assert np.array_equal(ia, ib)
    for f in ("e", "b"):
        ga = np.stack([a.fields[f].store(s) for s in range(1, d.nz + 1)])
        gb = np.stack([b.fields[f].store(s) for s in range(1, d.nz + 1)])
        assert store_errors(gb, ga).max() < tol
    a.close()
    b.close()


def test_batch_autotune_keeps_results():
    """The batch autotuner (cluster policy and iterations per loop body, timed on whole batch
    steps) leaves the simulations where they were: a batch step after it equals single steps
    of the same simulations (FP64: identical iteration counts, fields within 1e-9)."""
    decks = _decks()
    single = [Q.build_simulation(d) for d in decks]
    its_single = [s.run_3d_step()[0] for s in single]
    sims = [Q.build_simulation(d) for d in decks]
    batch = Q.Batch(sims)
    tune = batch.autotune(reps=1)
    assert tune["unroll"] in (1, 2, 4) and tune["step_ms"] > 0.0
    its_batch = batch.step()
    for d, a, b, ia, ib in zip(decks, single, sims, its_single, its_batch):
        assert np.array_equal(ia, ib), (d.name, ia, ib)
        for f in ("e", "b", "psi"):
            assert store_errors(b.fields[f].store_all(), a.fields[f].store_all()).max() < 1e-9, (d.name, f)
    batch.close()
    for s in single + sims:
        s.close()
