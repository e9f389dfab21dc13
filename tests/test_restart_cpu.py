"""Beam restart files (host side): names follow the reference's RST layout, the files are HDF5
in the reference's particle layout, and the particle arrays come back exactly (the beam
parameters come from the deck, as in the reference).  Stand-in objects replace the device
simulation, so this runs without a GPU."""
import numpy as np
import pytest

from qpad_gb300 import restart


class _Beam:
    def __init__(self, x, p, q, qbm, push_type, evolution, npmax):
        self.x, self.p, self.q = x, p, q
        self.qbm, self.push_type, self.evolution, self.npmax = qbm, push_type, evolution, npmax

    def download(self):
        return self.x, self.p, self.q


class _Sim:
    dt = 10.0

    def __init__(self):
        self.beams = []

    def add_beam(self, x, p, q, *, qbm, push_type, evolution, npmax):
        b = _Beam(np.array(x), np.array(p), np.array(q), qbm, push_type, evolution, npmax)
        self.beams.append(b)
        return b


def test_rst_path_matches_reference_names(tmp_path):
    path = restart.rst_path(str(tmp_path), 3, 120, rank=0)
    assert path.endswith("RST/Beam03/RST-beam03-000000_00000120.h5")


def test_save_load_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    src = _Sim()
    for k, n in enumerate((1000, 1)):
        src.add_beam(rng.standard_normal((n, 3)), rng.standard_normal((n, 3)), rng.standard_normal(n),
                     qbm=-1.0 / (k + 1), push_type=1 + k, evolution=bool(k), npmax=2 * n)
    paths = restart.save_beams(src, str(tmp_path), timestep=7)
    assert len(paths) == 2
    dst = _Sim()
    restart.load_beams(dst, str(tmp_path), timestep=7, nbeams=2,
                       params=[dict(qbm=b.qbm, push_type=b.push_type, evolution=b.evolution) for b in src.beams])
    for a, b in zip(src.beams, dst.beams):
        assert np.array_equal(a.x, b.x) and np.array_equal(a.p, b.p) and np.array_equal(a.q, b.q)
        assert (a.qbm, a.push_type, a.evolution) == (b.qbm, b.push_type, b.evolution)
        assert b.npmax >= len(b.q)
    with pytest.raises(FileNotFoundError):
        restart.load_beams(_Sim(), str(tmp_path), timestep=8, nbeams=1)


def test_rst_file_layout(tmp_path):
    """The file is the reference's particle file: root attribute tp and datasets x [n][3],
    p [n][3], q [n], read here by an independent parser of the format."""
    from tests import h5_parse
    rng = np.random.default_rng(2)
    src = _Sim()
    src.add_beam(rng.standard_normal((37, 3)), rng.standard_normal((37, 3)), rng.standard_normal(37), qbm=-1.0,
                 push_type=1, evolution=True, npmax=37)
    src.add_beam(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0), qbm=-1.0, push_type=1, evolution=True, npmax=1)
    p1, p2 = restart.save_beams(src, str(tmp_path), timestep=3)
    f = h5_parse.File(p1)
    assert f.attrs["tp"] == [37] and f.attrs["TYPE"].rstrip() == "restart" and f.attrs["ITER"] == [3]
    assert f.attrs["NAME"].rstrip() == "RST-beam01-000000" and f.attrs["TIME"] == [30.0]
    assert sorted(f.members()) == ["p", "q", "x"]
    assert np.array_equal(f.dataset("x"), src.beams[0].x) and np.array_equal(f.dataset("q"), src.beams[0].q)
    g = h5_parse.File(p2)
    assert g.attrs["tp"] == [0] and g.members() == []
    x, p, q = restart.read_rst(p2)
    assert len(q) == 0
