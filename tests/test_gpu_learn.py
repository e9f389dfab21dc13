"""The learned guess: GPU forward/backward of the conv net against the NumPy reference, GPU
training, the training samples against the 3D stores, and the guess in the slice loop."""
import numpy as np
import pytest

import qpad_gb300 as Q
from qpad_gb300 import learned as LR
from tests import nn_ref
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

SHAPE = dict(cin=3, cout=2, width=16, layers=3, K=5)


def _toy(seed, ns=4, nr=40):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((ns, SHAPE["cin"], nr)).astype(np.float32)
    t = rng.standard_normal((ns, SHAPE["cout"], nr)).astype(np.float32)
    net = LR.ConvNet(SHAPE["cin"], SHAPE["cout"], SHAPE["width"], SHAPE["layers"], SHAPE["K"], seed=seed)
    return net, x, t


def test_forward_matches_numpy():
    net, x, _ = _toy(1)
    p = net.get_params()
    y = net.predict(x)
    yr, _ = nn_ref.forward(p, x, **SHAPE)
    assert rel_l2(y, yr) < 2e-3


def test_gradient_matches_numpy():
    net, x, t = _toy(2)
    p = net.get_params()
    loss, g = net.grad(x, t)
    lr_, gr = nn_ref.loss_grad(p, x, t, **SHAPE)
    assert abs(loss - lr_) <= 2e-3 * abs(lr_)
    lay, _ = LR.layout(SHAPE["cin"], SHAPE["cout"], SHAPE["width"], SHAPE["layers"], SHAPE["K"])
    for wo, sh, bo in lay:                 # every layer's weights and biases
        n = int(np.prod(sh))
        assert rel_l2(g[wo:wo + n], gr[wo:wo + n]) < 2e-2, (wo, sh)
        assert rel_l2(g[bo:bo + sh[0]], gr[bo:bo + sh[0]]) < 2e-2, (bo, sh)


def test_training_reduces_loss():
    rng = np.random.default_rng(3)
    ns, nr = 64, 48
    x = rng.standard_normal((ns, SHAPE["cin"], nr)).astype(np.float32)
    k = np.array([0.25, 0.5, 0.25])
    t = np.stack([np.stack([np.convolve(x[s, 0] + 0.5 * x[s, 1], k, mode="same"),
                            np.tanh(x[s, 2])]) for s in range(ns)]).astype(np.float32)
    net = LR.ConvNet(SHAPE["cin"], SHAPE["cout"], SHAPE["width"], SHAPE["layers"], SHAPE["K"], seed=3)
    losses = net.train(x, t, epochs=60, batch=16, lr=3e-3, seed=3)
    assert losses[-1] < 0.1 * losses[0], losses


def _deck(M=1, nz=24, n_b=2.0, seed=3):
    return Q.decks.Deck("guess_test", nr=64, nz=nz, max_mode=M, dr=0.04, dxi=0.04, ppc=(2, 1), num_theta=8,
                        uth=2e-3, seed=seed, beams=[Q.decks.BeamSpec(n_b, 0.4, 0.3, 0.5, 20000, x0=0.04)],
                        iter_max=30, iter_reltol=1e-6)


def test_guess_samples_match_stores():
    deck = _deck()
    sim = Q.build_simulation(deck)
    sim.run_3d_step()
    b = np.stack([sim.b_spe.store(s) for s in range(1, deck.nz + 1)])
    cu = np.stack([sim.cu.store(s) for s in range(1, deck.nz + 1)])
    q = np.stack([sim.q_spe.store(s) for s in range(1, deck.nz + 1)])
    for m in (0, 1):
        parts = [0] if m == 0 else [1, 2]
        x, t, sc = LR.samples(sim, m, [5, 11])
        for k, j in enumerate([5, 11]):
            rows = []
            for d in (1, 2):
                s = j - d - 1
                for qq in range(5):
                    for p in parts:
                        if qq < 2:
                            rows.append(b[s, p, qq, 1:-1])
                        elif qq < 4:
                            rows.append(cu[s, p, qq - 2, 1:-1])
                        else:
                            rows.append(q[s, p, 0, 1:-1] - cu[s, p, 2, 1:-1])
            raw = np.array(rows)
            scale = np.sqrt(np.mean(raw ** 2))
            assert abs(sc[k] - scale) <= 1e-5 * scale
            assert rel_l2(x[k], raw / scale) < 1e-6
            tr = []
            for qq in range(4):
                for p in parts:
                    if qq < 2:      # what the linear extrapolation from slices j-1, j-2 misses
                        tr.append(b[j - 1, p, qq, 1:-1] - (2 * b[j - 2, p, qq, 1:-1] - b[j - 3, p, qq, 1:-1]))
                    else:
                        tr.append((cu[j - 1, p, qq - 2, 1:-1] - cu[j - 2, p, qq - 2, 1:-1]) / deck.dxi)
            assert rel_l2(t[k], np.array(tr) / scale) < 1e-5
    sim.close()


def test_guess_hook_with_zero_net_keeps_the_answer():
    deck = _deck()
    a = Q.build_simulation(deck)
    ia, _ = a.run_3d_step()
    b = Q.build_simulation(deck)
    n0, n1 = LR.ConvNet(*LR.CHANNELS[0]), LR.ConvNet(*LR.CHANNELS[1])
    n0.set_params(np.zeros(n0.nparam, np.float32))
    n1.set_params(np.zeros(n1.nparam, np.float32))
    LR.attach(b, n0, n1)
    ib, _ = b.run_3d_step()
    # the iteration still runs to iter_reltol from the different guess
    for s in range(1, deck.nz + 1, 5):
        assert rel_l2(b.e.store(s), a.e.store(s)) < 1e-4
        assert rel_l2(b.b.store(s), a.b.store(s)) < 1e-4
    assert abs(ib.mean() - ia.mean()) < 3.0
    LR.attach(b, None, None)
    a.close()
    b.close()


def test_zero_residual_net_is_the_linear_extrapolation():
    """The nets predict what the linear extrapolation of B-perp misses: nets that output zero
    give exactly the run with the linear extrapolation alone (qpad_set_guess_extrapolation 1)."""
    deck = _deck()
    a = Q.build_simulation(deck)
    a.set_guess_extrapolation(1)
    ia, _ = a.run_3d_step()
    b = Q.build_simulation(deck)
    n0, n1 = LR.ConvNet(*LR.CHANNELS[0]), LR.ConvNet(*LR.CHANNELS[1])
    n0.set_params(np.zeros(n0.nparam, np.float32))
    n1.set_params(np.zeros(n1.nparam, np.float32))
    LR.attach(b, n0, n1)
    ib, _ = b.run_3d_step()
    assert np.array_equal(ia, ib)
    for name in ("e", "b", "psi"):
        assert rel_l2(b.fields[name].store_all(), a.fields[name].store_all()) < 1e-12
    a.close()
    b.close()


def test_trained_guess_effect_on_iterations(record_property):
    """What the committed c2 guess nets change on a held-out c2-shaped driver (first 192
    slices): iterations per slice with and without them, and the fields still agree."""
    import os
    from qpad_gb300.train_guess import DEFAULT_OUT, c2_variant
    if not os.path.exists(DEFAULT_OUT):
        pytest.skip("no trained weights")
    net0, net1 = LR.load(DEFAULT_OUT, 2)
    d = c2_variant(3.0, 999, nz=192)
    a = Q.build_simulation(d, precision=Q._capi.PREC_MIXED)
    ia, _ = a.run_3d_step()
    b = Q.build_simulation(d, precision=Q._capi.PREC_MIXED)
    LR.attach(b, net0, net1)
    ib, _ = b.run_3d_step()
    record_property("iters_per_slice_plain", float(ia.mean()))
    record_property("iters_per_slice_guess", float(ib.mean()))
    print(f"iterations per slice: plain {ia.mean():.3f}, with the learned guess {ib.mean():.3f}")
    for s in range(8, d.nz + 1, 23):
        assert rel_l2(b.e.store(s), a.e.store(s)) < 2e-2
    assert ib.max() <= d.iter_max
    a.close()
    b.close()


@pytest.mark.parametrize("nr,M", [(150, 2), (64, 1), (40, 0)])
def test_fused_guess_matches_the_per_layer_forward(nr, M):
    """The guess kernel (the whole net of a radial tile in shared memory, one launch for every
    mode) against the nets' per-layer forward (qpad_learn_predict) on the same inputs: the
    extrapolated part to round-off, the nets' correction within the BF16 rounding of the
    activations; on ragged tiles (nr = 150 is two full tiles and a partial one)."""
    import ctypes as C
    d = Q.decks.Deck("guess_fused", nr=nr, nz=12, max_mode=M, dr=0.04, dxi=0.04, ppc=(2, 1), num_theta=8,
                     uth=2e-3, seed=4, beams=[Q.decks.BeamSpec(3.0, 0.4, 0.3, 0.4, 20000, x0=0.05)],
                     iter_max=30, iter_reltol=1e-6)
    sim = Q.build_simulation(d)
    sim.run_3d_step()
    nets = [LR.ConvNet(*LR.CHANNELS[0], seed=11), LR.ConvNet(*LR.CHANNELS[1], seed=12) if M >= 1 else None]
    for n in nets:                      # last layers at full scale, so the correction is not small
        if n is not None:
            p = n.get_params()
            n.set_params(p * np.float32(3.0))
    LR.attach(sim, *nets)
    LR.configure(sim, apply_b=True, apply_j=True)
    j = 7
    cu_before = sim.cu.download().copy()
    l0 = sim.launch_count()
    sim._check(sim.lib.qpad_guess_apply(sim.h, j))
    assert sim.launch_count() - l0 == 3        # slice index, inputs, the fused net
    b_got, cu_got = sim.b_spe.download(), sim.cu.download()
    b1, b2, cu1 = sim.b_spe.store(j - 1), sim.b_spe.store(j - 2), sim.cu.store(j - 1)
    for m in range(M + 1):
        parts = [0] if m == 0 else [2 * m - 1, 2 * m]
        nh = len(parts)
        x, _, sc = LR.samples(sim, m, [j])
        y = nets[0 if m == 0 else 1].predict(x)[0].astype(np.float64) * float(sc[0])
        for h, p in enumerate(parts):
            for c in range(2):
                ext = 2 * b1[p, c, 1:-1] - b2[p, c, 1:-1]
                want = ext + np.where(np.arange(nr) == 0, 0.0, y[c * nh + h])
                got = b_got[p, c, 1:-1]
                assert rel_l2(got[:1], ext[:1]) < 1e-12 or abs(got[0] - ext[0]) < 1e-14
                assert rel_l2(got - ext, want - ext) < 1e-2, (m, p, c)
                cj = cu1[p, c, 2:-1] + d.dxi * y[2 * nh + c * nh + h][1:]
                assert rel_l2(cu_got[p, c, 2:-1] - cu_before[p, c, 2:-1], cj - cu_before[p, c, 2:-1]) < 1e-2
    LR.attach(sim, None, None)
    sim.close()
