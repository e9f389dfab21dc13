"""The library's HDF5 files (field dumps and particle files in the reference's layout),
checked with an independent parser of the format and read back by the library's reader.
No GPU needed."""
import ctypes as C
import os

import numpy as np

from qpad_gb300 import _capi as K
from qpad_gb300.diagnostics import read_h5_attr, read_h5_dataset
from tests import h5_parse


def _grid_info(time=2.5, it=7, dt=0.5):
    info = K.H5GridInfo()
    info.time, info.iter, info.dt = time, it, dt
    info.timeunit, info.units, info.label = b"1 / \\omega_p", b"m_ec\\omega_p/e", b"E_z"
    info.axis_min[:] = [0.0, 0.0]
    info.axis_max[:] = [10.24, 5.12]
    info.axis_name[:] = [b"r", b"\\xi"]
    info.axis_label[:] = [b"r", b"\\xi"]
    info.axis_units[:] = [b"c / \\omega_p", b"c / \\omega_p"]
    return info


def test_grid_file_layout(tmp_path):
    L = K.load()
    rng = np.random.default_rng(0)
    data = np.ascontiguousarray(rng.standard_normal((24, 33)))
    path = os.path.join(str(tmp_path), "Fields", "Ez", "Re0", "ez_00000007.h5")
    assert L.qpad_h5_write_grid(path.encode(), b"ez", data.ctypes.data_as(K.D), 24, 33,
                                C.byref(_grid_info())) == 0
    f = h5_parse.File(path)
    # the reference's merge tool takes the second member of the root group as the data
    assert f.members() == ["AXIS", "ez"]
    a = f.attrs
    assert a["NAME"] == "ez".ljust(100) and a["TYPE"].rstrip() == "grid" and a["ITER"] == [7]
    assert a["TIME"] == [2.5] and a["DT"] == [0.5] and a["TIME UNIT"].rstrip() == "1 / \\omega_p"
    assert np.array_equal(f.dataset("ez"), data)
    ds = f.obj("ez")
    assert ds["attrs"]["UNITS"].rstrip() == "m_ec\\omega_p/e" and ds["attrs"]["LONG_NAME"].rstrip() == "E_z"
    assert f.members("AXIS") == ["AXIS1", "AXIS2"]
    assert f.dataset("AXIS/AXIS1").tolist() == [0.0, 10.24] and f.dataset("AXIS/AXIS2").tolist() == [0.0, 5.12]
    ax = f.obj("AXIS/AXIS2")["attrs"]
    assert ax == {"TYPE": "linear", "UNITS": "c / \\omega_p", "NAME": "\\xi", "LONG_NAME": "\\xi"}
    # the library's own reader
    assert np.array_equal(read_h5_dataset(path, "ez"), data)
    assert read_h5_dataset(path, "AXIS/AXIS1").tolist() == [0.0, 10.24]
    assert read_h5_attr(path, "ITER") == 7.0 and read_h5_attr(path, "TYPE") == "grid"
    assert read_h5_attr(path, "LONG_NAME", "ez") == "E_z"


def test_restart_grid_file_layout(tmp_path):
    """A grid restart file (a laser envelope part): TYPE "restart", no AXIS group
    (wrattr_file, hdf5io_class.f03:264-300)."""
    L = K.load()
    data = np.ascontiguousarray(np.arange(12.0).reshape(3, 4))
    path = os.path.join(str(tmp_path), "RST", "Laser01", "RST-laser01-re_re0_00000004.h5")
    info = _grid_info(it=4)
    info.type = b"restart"
    assert L.qpad_h5_write_grid(path.encode(), b"RST-laser01-re_re0", data.ctypes.data_as(K.D), 3, 4,
                                C.byref(info)) == 0
    f = h5_parse.File(path)
    assert f.members() == ["RST-laser01-re_re0"]
    assert f.attrs["TYPE"].rstrip() == "restart" and f.attrs["ITER"] == [4]
    assert np.array_equal(f.dataset("RST-laser01-re_re0"), data)
    assert np.array_equal(read_h5_dataset(path, "RST-laser01-re_re0").reshape(3, 4), data)


def test_particle_file_layout(tmp_path):
    L = K.load()
    rng = np.random.default_rng(1)
    n = 1000
    x, p, q = rng.standard_normal((n, 3)), rng.standard_normal((n, 3)), rng.standard_normal(n)
    path = os.path.join(str(tmp_path), "RST", "Beam01", "RST-beam01-000000_00000004.h5")
    assert L.qpad_h5_write_particles(path.encode(), b"RST-beam01-000000", x.ctypes.data_as(K.D),
                                     p.ctypes.data_as(K.D), q.ctypes.data_as(K.D), n, 4, 40.0, 10.0) == 0
    f = h5_parse.File(path)
    assert f.members() == ["p", "q", "x"] and f.attrs["tp"] == [n] and f.attrs["TYPE"].rstrip() == "restart"
    for name, arr in (("x", x), ("p", p), ("q", q)):
        assert np.array_equal(f.dataset(name), arr)
        assert np.array_equal(read_h5_dataset(path, name), arr)


def test_reader_errors(tmp_path):
    bad = os.path.join(str(tmp_path), "bad.h5")
    open(bad, "wb").write(b"not hdf5" * 20)
    for call in (lambda: read_h5_dataset(bad, "x"), lambda: read_h5_dataset(os.path.join(str(tmp_path), "no.h5"), "x")):
        try:
            call()
        except IOError:
            continue
        raise AssertionError("expected an error")
