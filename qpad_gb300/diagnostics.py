"""Diagnostics of a 3D step: the per-mode field error between two runs of the same inputs.

The error measure is the one the benchmark metric is quoted with ("... @1e-4 err"): for each
field, azimuthal mode m and component, the relative L2 norm of the difference over the whole
3D step (every slice, nodes 1..nr and the outer guard), the Re and Im parts of a mode taken
together as one complex amplitude.  Modes whose reference norm is below 1e-6 of the
component's norm over all modes hold round-off only (for instance the odd modes of an axially
symmetric case) and are not rated.  The slice contributing most to the squared error is
reported beside each figure.
"""
from __future__ import annotations

import numpy as np

# the fields whose 3D stores the step writes and the error covers: psi, E, B, J, rho
ERROR_FIELDS = ("psi", "e", "b", "cu", "q_spe")


def mode_errors(got: np.ndarray, ref: np.ndarray, max_mode: int, floor: float = 1e-6) -> dict:
    """{(m, component): (relative L2 error, worst slice 1-based, its share of the squared
    error)} for two stores shaped (nz, P, ncomp, nr+2)."""
    out = {}
    for m in range(max_mode + 1):
        parts = [0] if m == 0 else [2 * m - 1, 2 * m]
        for c in range(ref.shape[2]):
            r = ref[:, parts, c, 1:]
            nrm = float(np.linalg.norm(r))
            if not nrm > floor * float(np.linalg.norm(ref[:, :, c, 1:])):
                continue
            d = got[:, parts, c, 1:] - r
            per = np.einsum("spi,spi->s", d, d)
            tot = float(per.sum())
            s = int(np.argmax(per))
            out[(m, c)] = (float(np.sqrt(tot)) / nrm, s + 1, float(per[s] / tot) if tot > 0 else 0.0)
    return out


def step_error_report(got: dict, ref: dict, max_mode: int) -> dict:
    """Per-mode errors of every field in both dicts {field name: store}; returns
    {"max": worst error, "worst": "field[c] m=..", "worst_slice": s, "per_mode": {...}}."""
    per = {}
    for name in ERROR_FIELDS:
        if name not in got or name not in ref:
            continue
        for (m, c), v in mode_errors(got[name], ref[name], max_mode).items():
            per[f"{name}[{c}] m={m}"] = v
    if not per:
        return {"max": None, "worst": None, "worst_slice": None, "per_mode": {}}
    key = max(per, key=lambda k: per[k][0])
    return {"max": per[key][0], "worst": key, "worst_slice": per[key][1],
            "per_mode": {k: float(f"{v[0]:.4g}") for k, v in per.items()}}


def fp32_state(pl, dr):
    """The plasma arrays (x, p, gamma, psi, q) rounded as the mixed path holds them (integer
    cell + FP32 offset per coordinate, FP32 momenta, gamma, psi and charge), back in FP64.
    An FP64 run from these inputs differs from one from the originals only by the rounding
    of the initial state: the deck's own sensitivity to FP32 particle state."""
    x, p, g, ps, q = pl
    t = x * (1.0 / dr)
    s = np.floor(t)
    f = (t - s).astype(np.float32)
    up = f >= np.float32(1.0)
    f[up] -= np.float32(1.0)
    s[up] += 1.0
    xr = np.ascontiguousarray((s + f.astype(np.float64)) * dr)

    def r32(a):
        return np.ascontiguousarray(np.asarray(a).astype(np.float32).astype(np.float64))
    return xr, r32(p), r32(g), r32(ps), r32(q)
