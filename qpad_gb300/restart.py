"""Beam restart files: the only checkpoint state of a run (plasma is re-injected every 3D step).

Follows the reference's RST output and input (diagnostics_class.f03:696-717 writes,
sim_beams_class.f03:121-128 reads at start-up with `simulation.restart_timestep`,
part3d_class.f03:827-865 `writerst` / `readrst`): per beam i (1-based) a file under
``RST/Beam<ii>/`` named ``RST-beam<ii>-<rank, 6 digits>_<time step, 8 digits>`` holding the
beam's particles x (n, 3), p (n, 3), q (n) and their count.  The reference writes HDF5; no
HDF5 library is available here, so the same arrays go into a NumPy archive (``.npz``) with
the beam's creation parameters beside them, enough to re-create it on the device.
"""
from __future__ import annotations

import os

import numpy as np


def rst_path(root: str, beam: int, timestep: int, rank: int = 0) -> str:
    """File of beam `beam` (1-based) at 3D step `timestep`."""
    return os.path.join(root, "RST", f"Beam{beam:02d}", f"RST-beam{beam:02d}-{rank:06d}_{timestep:08d}.npz")


def save_beams(sim, root: str, timestep: int, rank: int = 0) -> list[str]:
    """Downloads every beam of `sim` from the device and writes its restart file; returns the
    paths."""
    paths = []
    for i, bm in enumerate(sim.beams, start=1):
        x, p, q = bm.download()
        path = rst_path(root, i, timestep, rank)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "wb") as f:
            np.savez(f, x=np.asarray(x, np.float64), p=np.asarray(p, np.float64), q=np.asarray(q, np.float64),
                     npp=np.int64(len(q)), qbm=np.float64(bm.qbm), push_type=np.int32(bm.push_type),
                     evolution=np.int32(bm.evolution), npmax=np.int64(bm.npmax or len(q)),
                     timestep=np.int64(timestep))
        paths.append(path)
    return paths


def load_beams(sim, root: str, timestep: int, nbeams: int, rank: int = 0, params: list | None = None) -> list:
    """Re-creates beams 1..nbeams on `sim` from their restart files at `timestep` (the
    reference's read_restart start-up); returns the new beams.  `params[i]` (qbm, push_type,
    evolution), when given, overrides what the file recorded: the reference takes them from
    the input deck and only the particles from the file."""
    out = []
    for i in range(1, nbeams + 1):
        path = rst_path(root, i, timestep, rank)
        if not os.path.exists(path):
            raise FileNotFoundError(f"no restart file for beam {i} at step {timestep}: {path}")
        with np.load(path) as d:
            n = int(d["npp"])
            x, p, q = d["x"][:n], d["p"][:n], d["q"][:n]
            kw = dict(qbm=float(d["qbm"]), push_type=int(d["push_type"]), evolution=bool(int(d["evolution"])))
            if params is not None:
                kw.update(params[i - 1])
            out.append(sim.add_beam(x, p, q, npmax=max(int(d["npmax"]), n, 1), **kw))
    return out
