"""Learned predictor-corrector guess: the conv nets, their training data and training.

A net per mode group maps the previous two slices' B-perp, J-perp and rho - Jz of one
azimuthal mode (over the radial nodes) to the increment of B-perp and to dJ-perp/dxi for
the next slice (``qpad_guess_sample`` in include/qpad_gpu.h fixes the channels and their
normalisation).  Net ``m0`` serves m = 0 (10 -> 4 channels), net ``m1`` every m >= 1
(20 -> 8 channels).  Forward, backward and Adam run in the library's own kernels
(csrc/learn.cu); this module only moves host arrays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _capi as K
from .api import QpadError, Simulation

WIDTH, LAYERS, KSIZE = 64, 4, 5
CHANNELS = {0: (10, 4), 1: (20, 8)}     # mode group -> (inputs, outputs)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class ConvNet:
    """A radial 1D conv net (conv1d(ksize) x layers, GELU between) on the GPU."""

    def __init__(self, cin, cout, width=WIDTH, layers=LAYERS, ksize=KSIZE, seed=0, device=0):
        self.lib = K.load()
        h = C.c_void_p()
        r = self.lib.qpad_learn_create(cin, cout, width, layers, ksize, seed, device, C.byref(h))
        if r != 0:
            raise QpadError(f"qpad_learn_create failed ({r})")
        self.h, self.cin, self.cout = h, cin, cout
        self.shape = (cin, cout, width, layers, ksize)

    def _check(self, r):
        if r != 0:
            raise QpadError(f"learn error {r}: {self.lib.qpad_learn_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.qpad_learn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nparam(self) -> int:
        n = C.c_int64()
        self._check(self.lib.qpad_learn_param_count(self.h, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.nparam, np.float32)
        self._check(self.lib.qpad_learn_get_params(self.h, _fp(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparam
        self._check(self.lib.qpad_learn_set_params(self.h, _fp(p)))

    def predict(self, x: np.ndarray) -> np.ndarray:
        """x: [samples][cin][nr] -> [samples][cout][nr]."""
        x = np.ascontiguousarray(x, np.float32)
        ns, _, nr = x.shape
        y = np.zeros((ns, self.cout, nr), np.float32)
        self._check(self.lib.qpad_learn_predict(self.h, _fp(x), ns, nr, _fp(y)))
        return y

    def grad(self, x: np.ndarray, t: np.ndarray):
        """(mean squared error, its gradient w.r.t. the flat parameter vector)."""
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        ns, _, nr = x.shape
        loss = C.c_double()
        g = np.zeros(self.nparam, np.float32)
        self._check(self.lib.qpad_learn_grad(self.h, _fp(x), _fp(t), ns, nr, C.byref(loss), _fp(g)))
        return loss.value, g

    def train(self, x, t, epochs=10, batch=64, lr=1e-3, seed=0) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        ns, _, nr = x.shape
        losses = np.zeros(epochs)
        self._check(self.lib.qpad_learn_train(self.h, _fp(x), _fp(t), ns, nr, epochs, batch, lr, seed,
                                              losses.ctypes.data_as(C.POINTER(C.c_double))))
        return losses


def layout(cin, cout, width=WIDTH, layers=LAYERS, ksize=KSIZE):
    """[(weight offset, weight shape (co, ci, k), bias offset)] of the flat parameter vector."""
    out, off = [], 0
    for l in range(layers):
        ci = cin if l == 0 else width
        co = cout if l == layers - 1 else width
        out.append((off, (co, ci, ksize), off + co * ci * ksize))
        off += co * ci * ksize + co
    return out, off


def samples(sim: Simulation, m: int, j_range=None):
    """Training samples of mode m from the 3D stores of the simulation's last step:
    (x [n][cin][nr], t [n][cout][nr], scale [n])."""
    lib = sim.lib
    cin, cout = CHANNELS[0 if m == 0 else 1]
    js = list(j_range) if j_range is not None else list(range(3, sim.nz + 1))
    xs = np.zeros((len(js), cin, sim.nr), np.float32)
    ts = np.zeros((len(js), cout, sim.nr), np.float32)
    sc = np.zeros(len(js), np.float32)
    if js and js == list(range(js[0], js[-1] + 1)):      # a contiguous range: one call
        sim._check(lib.qpad_guess_samples(sim.h, js[0], js[-1], m, _fp(xs), _fp(ts), _fp(sc)))
        return xs, ts, sc
    for k, j in enumerate(js):
        s = C.c_float()
        sim._check(lib.qpad_guess_sample(sim.h, j, m, _fp(xs[k]), _fp(ts[k]), C.byref(s)))
        sc[k] = s.value
    return xs, ts, sc


def dataset(sim: Simulation, j_range=None):
    """All samples of one finished 3D step, grouped as the nets take them."""
    x0, t0, _ = samples(sim, 0, j_range)
    if sim.max_mode < 1:
        return (x0, t0), None
    parts = [samples(sim, m, j_range) for m in range(1, sim.max_mode + 1)]
    x1 = np.concatenate([p[0] for p in parts])
    t1 = np.concatenate([p[1] for p in parts])
    return (x0, t0), (x1, t1)


def attach(sim: Simulation, net0: ConvNet | None, net1: ConvNet | None):
    """Make the nets the initial guess of every slice j >= 3 of sim (None detaches)."""
    sim._check(sim.lib.qpad_guess_attach(sim.h, net0.h if net0 is not None else None,
                                         net1.h if net1 is not None else None))
    sim._guess_nets = (net0, net1)     # keep them alive while attached


def configure(sim: Simulation, apply_b=True, apply_j=True, weight=1.0):
    """Which parts of the attached guess are used, and the weight of the net's correction."""
    sim._check(sim.lib.qpad_guess_config(sim.h, int(apply_b) | (2 * int(apply_j)), float(weight)))


WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")


def weights_path(max_mode: int) -> str:
    """Trained weights for simulations with `max_mode` modes: guess_c5.npz (trained on
    c5-shaped runs, M = 4) for M > 2 when it exists, else guess_c2.npz (trained on c2-shaped
    runs, M = 2).  The m >= 1 net takes one mode at a time, so it serves any number of modes."""
    c5 = os.path.join(WEIGHTS, "guess_c5.npz")
    return c5 if max_mode > 2 and os.path.exists(c5) else os.path.join(WEIGHTS, "guess_c2.npz")


def save(path, net0: ConvNet, net1: ConvNet | None):
    d = {"p0": net0.get_params()}
    if net1 is not None:
        d["p1"] = net1.get_params()
    np.savez_compressed(path, **d)


def load(path, max_mode: int, device=0):
    z = np.load(path)
    net0 = ConvNet(*CHANNELS[0], device=device)
    net0.set_params(z["p0"])
    net1 = None
    if max_mode >= 1:
        net1 = ConvNet(*CHANNELS[1], device=device)
        net1.set_params(z["p1"])
    return net0, net1
