"""Shared helpers for the parity tests: seeded inputs and field comparisons."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O


def rel_l2(a: np.ndarray, b: np.ndarray, floor: float = 0.0) -> float:
    """||a - b|| / max(||b||, floor)."""
    d = float(np.linalg.norm((a - b).ravel()))
    n = max(float(np.linalg.norm(b.ravel())), floor)
    if n == 0.0:
        return d
    return d / n


def field_errors(gpu: np.ndarray, ref: np.ndarray, nodes=slice(1, None), floor_rel=1e-12):
    """Per (part, component) relative L2 over nodes 1..nr (+guard) of one slice field;
    parts/components whose reference norm is below floor_rel of the whole field's norm
    are compared against that floor instead of themselves."""
    P, nc = ref.shape[0], ref.shape[1]
    glob = float(np.linalg.norm(ref[:, :, nodes])) or 1.0
    errs = np.zeros((P, nc))
    for p in range(P):
        for c in range(nc):
            errs[p, c] = rel_l2(gpu[p, c, nodes], ref[p, c, nodes], floor=floor_rel * glob)
    return errs


def store_errors(gpu: np.ndarray, ref: np.ndarray, nodes=slice(1, None), floor_rel=1e-6):
    """Per (part, component) relative L2 of a whole 3D store, shape (nz, P, ncomp, nr+2),
    over all slices and nodes 1..nr (+guard).

    The norm is taken over the step, not slice by slice: ahead of the beam the plasma is
    neutral and psi holds round-off only, which summation order alone changes completely.
    Parts below floor_rel of the store's norm (round-off parts, e.g. the m>=1 parts of a
    ring loaded at evenly spaced angles) are compared against that floor."""
    P, nc = ref.shape[1], ref.shape[2]
    glob = float(np.linalg.norm(ref[:, :, :, nodes])) or 1.0
    errs = np.zeros((P, nc))
    for p in range(P):
        for c in range(nc):
            errs[p, c] = rel_l2(gpu[:, p, c, nodes], ref[:, p, c, nodes], floor=floor_rel * glob)
    return errs


def smooth_field(rng, g, ncomp, scale=1.0, zero_guards=True):
    """A smooth random slice field (sum of radial Gaussians) of shape (P, ncomp, nr+2)."""
    P = 2 * g.max_mode + 1
    r = np.arange(g.nr + 2) * g.dr - g.dr     # node i at r = (i-1) dr
    f = np.zeros((P, ncomp, g.nr + 2))
    R = g.nr * g.dr
    for p in range(P):
        for c in range(ncomp):
            for _ in range(3):
                a = rng.normal() * scale
                r0 = rng.uniform(0.0, 0.7 * R)
                w = rng.uniform(0.05, 0.3) * R
                f[p, c] += a * np.exp(-((r - r0) / w) ** 2)
    if zero_guards:
        f[:, :, 0] = 0.0
        f[:, :, -1] = 0.0
    return f


def plasma_to_oracle(x, p, gamma, psi, q) -> O.Plasma:
    pl = O.Plasma(len(q))
    pl.x[:] = x[:, 0]
    pl.y[:] = x[:, 1]
    pl.px[:] = p[:, 0]
    pl.py[:] = p[:, 1]
    pl.pz[:] = p[:, 2]
    pl.gamma[:] = gamma
    pl.psi[:] = psi
    pl.q[:] = q
    return pl


def beam_to_oracle(x, p, q) -> O.Beam:
    bm = O.Beam(len(q))
    bm.x[:], bm.y[:], bm.z[:] = x[:, 0], x[:, 1], x[:, 2]
    bm.px[:], bm.py[:], bm.pz[:] = p[:, 0], p[:, 1], p[:, 2]
    bm.q[:] = q
    return bm


def sorted_rows(*cols):
    """Rows of the given columns sorted lexicographically (multiset comparison)."""
    a = np.stack(cols, axis=1)
    idx = np.lexsort(a.T[::-1])
    return a[idx]
