"""Beam restart files: the only checkpoint state of a run (plasma is re-injected every 3D step).

Follows the reference's RST output and input (diagnostics_class.f03:696-717 names them,
sim_beams_class.f03:121-128 reads them at start-up with `simulation.restart_timestep`,
part3d_class.f03:827-865 `writerst` / `readrst` through hdf5io_class.f03:1584-1819): per
beam i (1-based) an HDF5 file ``RST/Beam<ii>/RST-beam<ii>-<rank, 6 digits>_<time step, 8
digits>.h5`` holding the root attribute ``tp`` (the particle count) and the datasets x [n][3],
p [n][3], q [n].  The files are written and read by the library's own HDF5 implementation, so
files of either program are read by the other.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np


def rst_name(beam: int, rank: int = 0) -> str:
    """The reference's data name of beam `beam`'s restart file."""
    return f"RST-beam{beam:02d}-{rank:06d}"


def rst_path(root: str, beam: int, timestep: int, rank: int = 0) -> str:
    """File of beam `beam` (1-based) at 3D step `timestep`."""
    return os.path.join(root, "RST", f"Beam{beam:02d}", f"{rst_name(beam, rank)}_{timestep:08d}.h5")


def _lib():
    from . import _capi as K
    return K, K.load()


def save_beams(sim, root: str, timestep: int, rank: int = 0) -> list[str]:
    """Downloads every beam of `sim` from the device and writes its restart file; returns the
    paths."""
    K, L = _lib()
    paths = []
    for i, bm in enumerate(sim.beams, start=1):
        x, p, q = (np.ascontiguousarray(a, np.float64) for a in bm.download())
        path = rst_path(root, i, timestep, rank)
        r = L.qpad_h5_write_particles(path.encode(), rst_name(i, rank).encode(), x.ctypes.data_as(K.D),
                                      p.ctypes.data_as(K.D), q.ctypes.data_as(K.D), len(q), int(timestep),
                                      float(timestep * sim.dt), float(sim.dt))
        if r:
            raise IOError(L.qpad_h5_last_error().decode())
        paths.append(path)
    return paths


def read_rst(path: str):
    """(x [n][3], p [n][3], q [n]) of one restart file."""
    K, L = _lib()
    n = C.c_int64()
    if L.qpad_rst_read(path.encode(), None, None, None, 0, C.byref(n)):
        raise IOError(L.qpad_h5_last_error().decode())
    m = max(n.value, 1)
    x, p, q = np.zeros((m, 3)), np.zeros((m, 3)), np.zeros(m)
    if L.qpad_rst_read(path.encode(), x.ctypes.data_as(K.D), p.ctypes.data_as(K.D), q.ctypes.data_as(K.D), m,
                       C.byref(n)):
        raise IOError(L.qpad_h5_last_error().decode())
    return x[:n.value], p[:n.value], q[:n.value]


def load_beams(sim, root: str, timestep: int, nbeams: int, rank: int = 0, params: list | None = None) -> list:
    """Re-creates beams 1..nbeams on `sim` from their restart files at `timestep` (the
    reference's read_restart start-up); returns the new beams.  The files hold particles
    only: `params[i]` (qbm, push_type, evolution) come from the input deck, as in the
    reference (default: an electron beam with the reduced pusher, evolving)."""
    out = []
    for i in range(1, nbeams + 1):
        path = rst_path(root, i, timestep, rank)
        if not os.path.exists(path):
            raise FileNotFoundError(f"no restart file for beam {i} at step {timestep}: {path}")
        x, p, q = read_rst(path)
        kw = dict(qbm=-1.0, push_type=1, evolution=True)
        if params is not None:
            kw.update(params[i - 1])
        out.append(sim.add_beam(np.ascontiguousarray(x), np.ascontiguousarray(p), np.ascontiguousarray(q),
                                npmax=max(len(q), 1), **kw))
    return out
