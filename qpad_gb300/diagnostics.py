"""Diagnostics of a 3D step: the per-mode field error between two runs of the same inputs.

The error measure is the one the benchmark metric is quoted with ("... @1e-4 err"): for each
field, azimuthal mode m and component, the relative L2 norm of the difference over the whole
3D step (every slice, nodes 1..nr and the outer guard), the Re and Im parts of a mode taken
together as one complex amplitude.  Modes whose reference norm is below 1e-6 of the
component's norm over all modes hold round-off only (for instance the odd modes of an axially
symmetric case) and are not rated.  The slice contributing most to the squared error is
reported beside each figure.  Beside the per-mode figure, the same error relative to the
component's norm over all modes says how large it is in the field itself: a mode that holds
only particle noise can carry an O(1) relative error that is a tiny part of the field.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# the fields whose 3D stores the step writes and the error covers: psi, E, B, J, rho
ERROR_FIELDS = ("psi", "e", "b", "cu", "q_spe")


def mode_errors(got: np.ndarray, ref: np.ndarray, max_mode: int, floor: float = 1e-6) -> dict:
    """{(m, component): (relative L2 error, worst slice 1-based, its share of the squared
    error, the error relative to the component's norm over all modes)} for two stores
    shaped (nz, P, ncomp, nr+2)."""
    out = {}
    for m in range(max_mode + 1):
        parts = [0] if m == 0 else [2 * m - 1, 2 * m]
        for c in range(ref.shape[2]):
            r = ref[:, parts, c, 1:]
            nrm = float(np.linalg.norm(r))
            nrm_all = float(np.linalg.norm(ref[:, :, c, 1:]))
            if not nrm > floor * nrm_all:
                continue
            d = got[:, parts, c, 1:] - r
            per = np.einsum("spi,spi->s", d, d)
            tot = float(per.sum())
            s = int(np.argmax(per))
            out[(m, c)] = (float(np.sqrt(tot)) / nrm, s + 1, float(per[s] / tot) if tot > 0 else 0.0,
                           float(np.sqrt(tot)) / nrm_all)
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
        return {"max": None, "worst": None, "worst_slice": None, "per_mode": {}, "max_vs_field": None,
                "worst_vs_field": None}
    key = max(per, key=lambda k: per[k][0])
    kf = max(per, key=lambda k: per[k][3])
    return {"max": per[key][0], "worst": key, "worst_slice": per[key][1],
            "per_mode": {k: float(f"{v[0]:.4g}") for k, v in per.items()},
            "max_vs_field": per[kf][3], "worst_vs_field": kf,
            "per_mode_vs_field": {k: float(f"{v[3]:.4g}") for k, v in per.items()}}


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


# ---- field dumps in the reference's layout ------------------------------------------------
# The reference's field diagnostics (field.diag names, diagnostics_class.f03:421-600): diag
# name -> (field object, component, directory under Fields/, data name, units, label).
FIELD_DIAGS = {
    "er_cyl_m": ("e", 0, "Er", "er", "m_ec\\omega_p/e", "E_r"),
    "ephi_cyl_m": ("e", 1, "Ephi", "ephi", "m_ec\\omega_p/e", "E_\\phi"),
    "ez_cyl_m": ("e", 2, "Ez", "ez", "m_ec\\omega_p/e", "E_z"),
    "br_cyl_m": ("b", 0, "Br", "br", "m_e\\omega_p/e", "B_r"),
    "bphi_cyl_m": ("b", 1, "Bphi", "bphi", "m_e\\omega_p/e", "B_\\phi"),
    "bz_cyl_m": ("b", 2, "Bz", "bz", "m_e\\omega_p/e", "B_z"),
    "spec_er_cyl_m": ("e_spe", 0, "Er_spec", "er", "m_ec\\omega_p/e", "E_r"),
    "spec_ephi_cyl_m": ("e_spe", 1, "Ephi_spec", "ephi", "m_ec\\omega_p/e", "E_\\phi"),
    "spec_ez_cyl_m": ("e_spe", 2, "Ez_spec", "ez", "m_ec\\omega_p/e", "E_z"),
    "spec_br_cyl_m": ("b_spe", 0, "Br_spec", "br", "m_e\\omega_p/e", "B_r"),
    "spec_bphi_cyl_m": ("b_spe", 1, "Bphi_spec", "bphi", "m_e\\omega_p/e", "B_\\phi"),
    "spec_bz_cyl_m": ("b_spe", 2, "Bz_spec", "bz", "m_e\\omega_p/e", "B_z"),
    "charge_cyl_m": ("q_spe", 0, "Charge", "charge", "n_0", "\\rho"),
    "jr_cyl_m": ("cu", 0, "Jr", "jr", "n_0 c", "J_r"),
    "jphi_cyl_m": ("cu", 1, "Jphi", "jphi", "n_0 c", "J_\\phi"),
    "jz_cyl_m": ("cu", 2, "Jz", "jz", "n_0 c", "J_z"),
    "psi_cyl_m": ("psi", 0, "Psi", "psi", "m_ec^2/e", "\\Psi"),
}


def mode_dirs(max_mode: int) -> list:
    """Per-part directories of a real field dump: Re0, Re1, Im1, ... (add_diag_cym)."""
    out = ["Re0"]
    for m in range(1, max_mode + 1):
        out += [f"Re{m}", f"Im{m}"]
    return out


def write_field_diags(sim, names, root: str, tstep: int) -> list:
    """The field dumps `names` (keys of FIELD_DIAGS) of the last 3D step into
    root/Fields/<Name>/<Re0|Re1|Im1|...>/<name>_<tstep, 8 digits>.h5 with TIME = tstep * dt;
    returns the directories written."""
    import os
    out = []
    for n in names:
        field, comp, sub, dataname, units, label = FIELD_DIAGS[n]
        d = os.path.join(root, "Fields", sub) + "/"
        f = sim.fields[field]
        sim._check(sim.lib.qpad_diag_write_field(sim.h, f.id, comp, d.encode(), dataname.encode(), units.encode(),
                                                 label.encode(), int(tstep), float(tstep * sim.dt), float(sim.dt)))
        out.append(d)
    return out


def read_h5_dataset(path: str, name: str):
    """A dataset of an HDF5 file (this library's reader) as a float64 array of its shape."""
    import ctypes as C

    from . import _capi as K
    L = K.load()
    n, rank = C.c_int64(), C.c_int32()
    dims = (C.c_int64 * 8)()
    if L.qpad_h5_read_dataset(path.encode(), name.encode(), None, 0, C.byref(n), C.byref(rank), dims):
        raise IOError(L.qpad_h5_last_error().decode())
    out = np.zeros(max(n.value, 1))
    if L.qpad_h5_read_dataset(path.encode(), name.encode(), out.ctypes.data_as(K.D), n.value, C.byref(n),
                              C.byref(rank), dims):
        raise IOError(L.qpad_h5_last_error().decode())
    return out[:n.value].reshape([dims[k] for k in range(rank.value)])


def read_h5_attr(path: str, attr: str, obj: str = ""):
    """An attribute (number or string, strings with the trailing padding removed)."""
    import ctypes as C

    from . import _capi as K
    L = K.load()
    v = C.c_double()
    buf = C.create_string_buffer(512)
    if L.qpad_h5_read_attr(path.encode(), obj.encode(), attr.encode(), C.byref(v), buf, 512):
        raise IOError(L.qpad_h5_last_error().decode())
    return buf.value.decode().rstrip() if buf.value else v.value


def laser_dirs(max_mode: int) -> list:
    """(directory, 0 for a_r / 1 for a_i, mode part) of a complex field dump (add_diag_cym,
    diagnostics_class.f03:1001-1015): Re_Re0, Im_Re0, then per mode Re_Re, Re_Im, Im_Re, Im_Im."""
    out = [("Re_Re0", 0, 0), ("Im_Re0", 1, 0)]
    for m in range(1, max_mode + 1):
        out += [(f"Re_Re{m}", 0, 2 * m - 1), (f"Re_Im{m}", 0, 2 * m), (f"Im_Re{m}", 1, 2 * m - 1),
                (f"Im_Im{m}", 1, 2 * m)]
    return out


def _grid_info(sim, tstep, units, label):
    from . import _capi as K
    info = K.H5GridInfo()
    info.time, info.iter, info.dt = float(tstep * sim.dt), int(tstep), float(sim.dt)
    info.timeunit, info.units, info.label = b"1 / \\omega_p", units.encode(), label.encode()
    info.axis_min[0], info.axis_max[0] = 0.0, sim.nr * sim.dr
    info.axis_min[1], info.axis_max[1] = 0.0, sim.nz * sim.dxi
    for k, n in enumerate((b"r", b"\\xi")):
        info.axis_name[k] = n
        info.axis_label[k] = n
        info.axis_units[k] = b"c / \\omega_p"
    return info


def write_laser_diags(sim, root: str, tstep: int, envelope: bool = True, chi: bool = True) -> list:
    """The laser dumps of the last 3D step (init_diag_lasers, diagnostics_class.f03:608-694):
    'a_cyl_m' of every laser i into root/Lasers<i>/A_laser/<Re_Re0|Im_Re0|...>/a_laser_<tstep>.h5
    and 'chi_cyl_m' into root/Fields/Chi/<Re0|Re1|Im1|...>/chi_<tstep>.h5; returns the files."""
    import os
    from . import _capi as K
    L = K.load()
    out = []

    def write(path, name, data, info):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = np.ascontiguousarray(data)
        if L.qpad_h5_write_grid(path.encode(), name.encode(), data.ctypes.data_as(K.D), sim.nz, sim.nr,
                                C.byref(info)):
            raise IOError(L.qpad_h5_last_error().decode())
        out.append(path)

    if envelope:
        info = _grid_info(sim, tstep, "m_ec^2/e", "a")
        for i, lz in enumerate(sim.lasers, start=1):
            arrs = lz.download()
            for d, h, p in laser_dirs(sim.max_mode):
                write(os.path.join(root, f"Lasers{i}", "A_laser", d, f"a_laser_{tstep:08d}.h5"), "a_laser",
                      arrs[h][:, p, 1:sim.nr + 1], info)
    if chi:
        info = _grid_info(sim, tstep, "n_0", "\\chi")
        c = sim.chi_store()
        for p, d in enumerate(mode_dirs(sim.max_mode)):
            write(os.path.join(root, "Fields", "Chi", d, f"chi_{tstep:08d}.h5"), "chi", c[:, p, 1:sim.nr + 1], info)
    return out
