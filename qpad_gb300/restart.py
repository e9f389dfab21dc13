"""Restart files: the beams and the laser envelopes, the checkpoint state of a run (plasma is
re-injected every 3D step).

Follows the reference's RST output and input (diagnostics_class.f03:696-717 names them,
sim_beams_class.f03:121-128 reads them at start-up with `simulation.restart_timestep`,
part3d_class.f03:827-865 `writerst` / `readrst` through hdf5io_class.f03:1584-1819): per
beam i (1-based) an HDF5 file ``RST/Beam<ii>/RST-beam<ii>-<rank, 6 digits>_<time step, 8
digits>.h5`` holding the root attribute ``tp`` (the particle count) and the datasets x [n][3],
p [n][3], q [n].  Per laser i an HDF5 grid file per mode part of a_r and a_i
(init_diag_rst_lasers, diagnostics_class.f03:719-742, add_diag_rst_laser :1087-1145; written by
field_complex::write_hdf5, field_complex_class.f03:833-863, read back by read_rst_field_laser,
field_laser_class.f03:1036-1058): ``RST/Laser<ii>/RST-laser<ii>-<part>_<time step, 8
digits>.h5`` with <part> re_re0, im_re0, then per mode m re_re<m>, re_im<m>, im_re<m>,
im_im<m> (a_r Re, a_r Im, a_i Re, a_i Im), the dataset of that name [nz][nr] and TYPE
"restart".  The files are written and read by the library's own HDF5 implementation, so
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


def laser_parts(max_mode: int) -> list:
    """(file part name, 0 for a_r / 1 for a_i, mode part) of a laser's restart files."""
    out = [("re_re0", 0, 0), ("im_re0", 1, 0)]
    for m in range(1, max_mode + 1):
        out += [(f"re_re{m}", 0, 2 * m - 1), (f"re_im{m}", 0, 2 * m), (f"im_re{m}", 1, 2 * m - 1),
                (f"im_im{m}", 1, 2 * m)]
    return out


def laser_rst_path(root: str, laser: int, part: str, timestep: int):
    """(file, data name) of laser `laser`'s (1-based) restart part at 3D step `timestep`."""
    name = f"RST-laser{laser:02d}-{part}"
    return os.path.join(root, "RST", f"Laser{laser:02d}", f"{name}_{timestep:08d}.h5"), name


def save_lasers(sim, root: str, timestep: int) -> list[str]:
    """Downloads every laser envelope of `sim` and writes its restart files; returns the paths."""
    K, L = _lib()
    paths = []
    info = K.H5GridInfo()
    info.time, info.iter, info.dt = float(timestep * sim.dt), int(timestep), float(sim.dt)
    info.timeunit, info.units, info.label, info.type = b"", b"", b"", b"restart"
    for k, lz in enumerate(sim.lasers, start=1):
        arrs = lz.download()
        for part, h, p in laser_parts(sim.max_mode):
            path, name = laser_rst_path(root, k, part, timestep)
            os.makedirs(os.path.dirname(path), exist_ok=True)
            data = np.ascontiguousarray(arrs[h][:, p, 1:sim.nr + 1])
            if L.qpad_h5_write_grid(path.encode(), name.encode(), data.ctypes.data_as(K.D), sim.nz, sim.nr,
                                    C.byref(info)):
                raise IOError(L.qpad_h5_last_error().decode())
            paths.append(path)
    return paths


def load_lasers(sim, root: str, timestep: int, nlasers: int, params: list) -> list:
    """Re-creates lasers 1..nlasers on `sim` from their restart files at `timestep`;
    params[i] = dict(k0=..., iteration=...) from the input deck (the files hold the envelope
    only).  Returns the new lasers."""
    from .diagnostics import read_h5_dataset
    out = []
    for k in range(1, nlasers + 1):
        ar = np.zeros((sim.nz, sim.P, sim.nr))
        ai = np.zeros((sim.nz, sim.P, sim.nr))
        for part, h, p in laser_parts(sim.max_mode):
            path, name = laser_rst_path(root, k, part, timestep)
            d = read_h5_dataset(path, name).reshape(sim.nz, sim.nr)
            (ar, ai)[h][:, p, :] = d
        out.append(sim.add_laser(ar, ai, **params[k - 1]))
    return out
