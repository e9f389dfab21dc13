"""ctypes binding of the CPU oracle (oracle/qpad_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
``bench.py``'s CPU-baseline leg, never by the product package.  Parity against the
reference itself is unpinned (see qpad_oracle.h); the oracle is pinned by the
project's own known-answer tests.

Arrays follow qpad_oracle.h: slice fields are float64 arrays shaped
``(P, ncomp, nr + 2)`` (P = 2M+1 mode parts, node index 0..nr+1), 3D stores are
``(nz + 1, P, ncomp, nr + 2)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libqpad_oracle.so")

D = C.POINTER(C.c_double)
I32 = C.POINTER(C.c_int32)


class Grid(C.Structure):
    _fields_ = [("nr", C.c_int), ("nz", C.c_int), ("max_mode", C.c_int), ("bnd", C.c_int),
                ("dr", C.c_double), ("dxi", C.c_double), ("relax_fac", C.c_double)]


class BeamDesc(C.Structure):
    _fields_ = [("tot_num", C.c_int64), ("tot_charge", C.c_double), ("qm", C.c_double),
                ("gamma", C.c_double), ("center", C.c_double * 3), ("sigma", C.c_double * 3),
                ("range_lo", C.c_double * 3), ("range_hi", C.c_double * 3),
                ("uth", C.c_double * 3), ("quiet", C.c_int)]


class Rng(C.Structure):
    _fields_ = [("s", C.c_uint64), ("have", C.c_int), ("next", C.c_double)]


class SimDesc(C.Structure):
    _fields_ = [("g", Grid), ("iter_max", C.c_int), ("iter_reltol", C.c_double),
                ("iter_abstol", C.c_double), ("dt3d", C.c_double), ("sp_qbm", C.c_double),
                ("sp_push_type", C.c_int), ("sp_neutralized", C.c_int), ("sp_npmax", C.c_int64),
                ("nbeams", C.c_int), ("beam_qbm", C.c_double * 4), ("beam_push_type", C.c_int * 4),
                ("beam_npmax", C.c_int64 * 4), ("nthreads", C.c_int), ("smooth_order", C.c_int),
                ("extrap", C.c_int), ("neut_levels", C.c_int), ("neut_adk", C.c_double * 48),
                ("neut_wp", C.c_double), ("neut_density", C.c_double), ("neut_ppc1", C.c_int),
                ("neut_ppc2", C.c_int), ("neut_num_theta", C.c_int), ("neut_qm", C.c_double),
                ("neut_qbm", C.c_double), ("neut_push_type", C.c_int), ("neut_npmax", C.c_int64),
                ("nlasers", C.c_int), ("laser_k0", C.c_double * 4), ("laser_iter", C.c_int * 4),
                ("sp_ppc_r", C.c_int)]


class LaserF1(C.Structure):
    _fields_ = [("ar", C.POINTER(C.c_double)), ("ai", C.POINTER(C.c_double)),
                ("gr", C.POINTER(C.c_double)), ("gi", C.POINTER(C.c_double))]


BND_ZERO, BND_OPEN = 2, 3
FK_PSI, FK_EZ, FK_BZ, FK_BT, FK_BPLUS, FK_BMINUS = range(6)
PUSH_STD, PUSH_ROBUST = 0, 1
PUSH_STD_PGC, PUSH_ROBUST_PGC = 4, 5
PUSH3_REDUCED, PUSH3_BORIS = 1, 2

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        G = C.POINTER(Grid)
        sig = {
            "orc_build_matrix": (None, [G, C.c_int, C.c_int, D, D, D]),
            "orc_thomas": (None, [C.c_int, D, D, D, D]),
            "orc_solve_psi": (None, [G, D, D]),
            "orc_solve_bz": (None, [G, D, D]),
            "orc_solve_bt_beam": (None, [G, D, D]),
            "orc_solve_bt_iter": (None, [G, D, D, D]),
            "orc_solve_ez": (None, [G, D, D]),
            "orc_solve_et": (None, [G, D, D, D]),
            "orc_solve_djdxi": (None, [G, D, D, D]),
            "orc_conv_record": (None, [G, D, D, D]),
            "orc_conv_compare": (None, [G, D, D, D, D, D]),
            "orc_qdeposit": (None, [G, C.c_int64, D, D, D, D]),
            "orc_smooth": (None, [G, C.c_int, D]),
            "orc_amjdeposit": (None, [G, C.c_int, C.c_double, C.c_double, C.c_int64, D, D, D, D, D, D,
                                      D, D, D, D, D, D, D, C.c_int]),
            "orc_push_u": (None, [G, C.c_int, C.c_double, C.c_double, C.c_int64, D, D, D, D, D, D, D,
                                  D, D, C.c_int]),
            "orc_push_x": (None, [C.c_int64, C.c_double, D, D, D, D, D, D]),
            "orc_update_bound": (C.c_int64, [G, C.c_int64, D, D, D, D, D, D, D, D]),
            "orc_interp_psi": (None, [G, C.c_int64, D, D, D, D]),
            "orc_sort": (None, [G, C.c_int64, D, D, D, D, D, D, D, D, I32, I32]),
            "orc_beam_qdeposit": (None, [G, C.c_int64, D, D, D, D, D]),
            "orc_beam_push": (None, [G, C.c_int, C.c_double, C.c_double, C.c_int64, D, D, D, D, D, D,
                                     D, D, C.c_int]),
            "orc_beam_update_bound": (C.c_int64, [G, C.c_int64, D, D, D, D, D, D, D]),
            "orc_rng_seed": (None, [C.POINTER(Rng), C.c_uint64]),
            "orc_rand_uniform": (C.c_double, [C.POINTER(Rng)]),
            "orc_rand_norm": (C.c_double, [C.POINTER(Rng)]),
            "orc_load_plasma": (C.c_int64, [G, C.POINTER(Rng), C.c_int, C.c_int, C.c_int, C.c_double,
                                            C.c_double, D, D, D, D, D, D, D, D, D]),
            "orc_load_beam": (C.c_int64, [G, C.POINTER(Rng), C.POINTER(BeamDesc), D, D, D, D, D, D, D]),
            "orc_sim_create": (C.c_void_p, [C.POINTER(SimDesc)]),
            "orc_sim_destroy": (None, [C.c_void_p]),
            "orc_sim_set_plasma": (None, [C.c_void_p, C.c_int64, D, D, D, D, D, D, D, D]),
            "orc_sim_set_beam": (None, [C.c_void_p, C.c_int, C.c_int64, D, D, D, D, D, D, D]),
            "orc_sim_run_3dstep": (None, [C.c_void_p, C.c_int, C.POINTER(C.c_int), D]),
            "orc_sim_begin_3dstep": (None, [C.c_void_p]),
            "orc_sim_slice": (None, [C.c_void_p, C.c_int, C.POINTER(C.c_int), D]),
            "orc_sim_end_3dstep": (None, [C.c_void_p, C.c_int]),
            "orc_sim_field": (D, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int)]),
            "orc_sim_store": (D, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int)]),
            "orc_sim_plasma": (C.c_int64, [C.c_void_p] + [C.POINTER(D)] * 8),
            "orc_sim_beam": (C.c_int64, [C.c_void_p, C.c_int] + [C.POINTER(D)] * 7),
            "orc_sim_neutral": (C.c_int64, [C.c_void_p] + [C.POINTER(D)] * 8),
            "orc_sim_multi_ion": (D, [C.c_void_p]),
            "orc_sim_set_laser": (None, [C.c_void_p, C.c_int, D, D]),
            "orc_sim_laser": (None, [C.c_void_p, C.c_int, C.POINTER(D), C.POINTER(D)]),
            "orc_pcr_coef": (None, [C.c_int, D, D, D, D, D, D, D, D, D, D]),
            "orc_pcr_solve": (None, [C.c_int, D, D, D, D, D, D]),
            "orc_laser_matrix": (None, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                        D, D, D, D, D]),
            "orc_laser_grad": (None, [C.POINTER(Grid), D, D, C.c_int, D, D]),
            "orc_deposit_chi": (None, [C.POINTER(Grid), C.c_double, C.c_int, C.c_int64, D, D, D, D, D]),
            "orc_amjdeposit_pgc": (None, [C.POINTER(Grid), C.c_int, C.c_double, C.c_double, C.c_int64] + [D] * 10
                                   + [C.POINTER(LaserF1), D, D, D]),
            "orc_push_u_pgc": (None, [C.POINTER(Grid), C.c_double, C.c_double, C.c_int64] + [D] * 9
                               + [C.POINTER(LaserF1)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def iptr(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(I32)


def laser_matrix(nr, m, k0, ds, dr, dz):
    """Rows (a, b, c, d, e) [5][2 nr] of the envelope's penta-diagonal system for mode m."""
    A = np.zeros((5, 2 * nr))
    lib().orc_laser_matrix(nr, m, k0, ds, dr, dz, *[ptr(A[k]) for k in range(5)])
    return A


def pcr_coef(A):
    """PCR tables of a penta-diagonal matrix A [5][n]: (cm1, cm2, cp1, cp2 [steps][n], cfin [n])."""
    n = A.shape[1]
    steps = int(np.ceil(np.log2(n)))
    A = np.ascontiguousarray(A, np.float64)
    c = [np.zeros((steps, n)) for _ in range(4)] + [np.zeros(n)]
    lib().orc_pcr_coef(n, *[ptr(A[k]) for k in range(5)], *[ptr(x) for x in c])
    return c


def pcr_solve(coef, rhs):
    x = np.ascontiguousarray(rhs, np.float64).copy()
    lib().orc_pcr_solve(len(x), *[ptr(c) for c in coef], ptr(x))
    return x


def grid(nr, nz, max_mode, dr, dxi, relax_fac=None, bnd=BND_OPEN) -> Grid:
    if relax_fac is None:
        relax_fac = 1.0e-3 * (dr / 0.02) ** 2      # sim_fields_class.f03:137-140
    return Grid(nr, nz, max_mode, bnd, dr, dxi, relax_fac)


def field(g: Grid, ncomp: int) -> np.ndarray:
    return np.zeros((2 * g.max_mode + 1, ncomp, g.nr + 2))


def store(g: Grid, ncomp: int) -> np.ndarray:
    return np.zeros((g.nz + 1, 2 * g.max_mode + 1, ncomp, g.nr + 2))


# ---- per-routine wrappers ------------------------------------------------------------

def build_matrix(g, kind, mode):
    a, b, c = (np.zeros(g.nr) for _ in range(3))
    lib().orc_build_matrix(C.byref(g), kind, mode, ptr(a), ptr(b), ptr(c))
    return a, b, c


def solve_psi(g, q):
    out = field(g, 1)
    lib().orc_solve_psi(C.byref(g), ptr(q), ptr(out))
    return out


def solve_bz(g, cu, b=None):
    b = field(g, 3) if b is None else b
    lib().orc_solve_bz(C.byref(g), ptr(cu), ptr(b))
    return b


def solve_bt_beam(g, q, b=None):
    b = field(g, 3) if b is None else b
    lib().orc_solve_bt_beam(C.byref(g), ptr(q), ptr(b))
    return b


def solve_bt_iter(g, dcu, cu, b):
    lib().orc_solve_bt_iter(C.byref(g), ptr(dcu), ptr(cu), ptr(b))
    return b


def solve_ez(g, cu, e=None):
    e = field(g, 3) if e is None else e
    lib().orc_solve_ez(C.byref(g), ptr(cu), ptr(e))
    return e


def solve_et(g, b, psi, e=None):
    e = field(g, 3) if e is None else e
    lib().orc_solve_et(C.byref(g), ptr(b), ptr(psi), ptr(e))
    return e


def solve_djdxi(g, acu, amu, dcu=None):
    dcu = field(g, 2) if dcu is None else dcu
    lib().orc_solve_djdxi(C.byref(g), ptr(acu), ptr(amu), ptr(dcu))
    return dcu


def conv_test(g, b_old, b_new):
    s_re, s_im = np.zeros(g.nr), np.zeros(g.nr)
    rel, ab = C.c_double(), C.c_double()
    lib().orc_conv_record(C.byref(g), ptr(b_old), ptr(s_re), ptr(s_im))
    lib().orc_conv_compare(C.byref(g), ptr(b_new), ptr(s_re), ptr(s_im), C.byref(rel), C.byref(ab))
    return rel.value, ab.value


class Plasma:
    """SoA plasma slice state (x, y, px, py, pz, gamma, psi, q) as float64 arrays."""
    NAMES = ("x", "y", "px", "py", "pz", "gamma", "psi", "q")

    def __init__(self, n):
        for k in self.NAMES:
            setattr(self, k, np.zeros(n))
        self.n = n

    def copy(self):
        o = Plasma(self.n)
        for k in self.NAMES:
            setattr(o, k, getattr(self, k).copy())
        return o

    def trim(self, n):
        o = Plasma(n)
        for k in self.NAMES:
            setattr(o, k, np.ascontiguousarray(getattr(self, k)[:n]))
        return o


def qdeposit(g, pl: Plasma, qf=None):
    qf = field(g, 1) if qf is None else qf
    lib().orc_qdeposit(C.byref(g), pl.n, ptr(pl.x), ptr(pl.y), ptr(pl.q), ptr(qf))
    return qf


def smooth(g, kind, f):
    """One smoothing pass in place (kind 0 rho, 1 jay, 2 djdxi)."""
    lib().orc_smooth(C.byref(g), kind, ptr(f))
    return f


def amjdeposit(g, push_type, qbm, dt, pl: Plasma, ef, bf, nthreads=1):
    cu, amu, dcu = field(g, 3), field(g, 3), field(g, 2)
    lib().orc_amjdeposit(C.byref(g), push_type, qbm, dt, pl.n, ptr(pl.x), ptr(pl.y), ptr(pl.px),
                         ptr(pl.py), ptr(pl.pz), ptr(pl.q), ptr(pl.gamma), ptr(pl.psi), ptr(ef),
                         ptr(bf), ptr(cu), ptr(amu), ptr(dcu), nthreads)
    return cu, amu, dcu


def push_u(g, push_type, qbm, dt, pl: Plasma, ef, bf, nthreads=1):
    lib().orc_push_u(C.byref(g), push_type, qbm, dt, pl.n, ptr(pl.x), ptr(pl.y), ptr(pl.px),
                     ptr(pl.py), ptr(pl.pz), ptr(pl.gamma), ptr(pl.psi), ptr(ef), ptr(bf), nthreads)


def push_x(pl: Plasma, dt):
    lib().orc_push_x(pl.n, dt, ptr(pl.x), ptr(pl.y), ptr(pl.px), ptr(pl.py), ptr(pl.pz), ptr(pl.gamma))


def update_bound(g, pl: Plasma) -> int:
    n = lib().orc_update_bound(C.byref(g), pl.n, ptr(pl.x), ptr(pl.y), ptr(pl.px), ptr(pl.py),
                               ptr(pl.pz), ptr(pl.gamma), ptr(pl.psi), ptr(pl.q))
    return int(n)


def interp_psi(g, pl: Plasma, psif):
    lib().orc_interp_psi(C.byref(g), pl.n, ptr(pl.x), ptr(pl.y), ptr(psif), ptr(pl.psi))


def sort(g, pl: Plasma):
    keys = np.zeros(pl.n, np.int32)
    idx = np.zeros(pl.n, np.int32)
    lib().orc_sort(C.byref(g), pl.n, ptr(pl.x), ptr(pl.y), ptr(pl.px), ptr(pl.py), ptr(pl.pz),
                   ptr(pl.gamma), ptr(pl.psi), ptr(pl.q), iptr(keys), iptr(idx))
    return keys, idx


class Beam:
    NAMES = ("x", "y", "z", "px", "py", "pz", "q")

    def __init__(self, n):
        for k in self.NAMES:
            setattr(self, k, np.zeros(n))
        self.n = n

    def copy(self):
        o = Beam(self.n)
        for k in self.NAMES:
            setattr(o, k, getattr(self, k).copy())
        return o

    def trim(self, n):
        o = Beam(n)
        for k in self.NAMES:
            setattr(o, k, np.ascontiguousarray(getattr(self, k)[:n]))
        return o


def beam_qdeposit(g, bm: Beam, q2=None):
    q2 = store(g, 1) if q2 is None else q2
    lib().orc_beam_qdeposit(C.byref(g), bm.n, ptr(bm.x), ptr(bm.y), ptr(bm.z), ptr(bm.q), ptr(q2))
    return q2


def beam_push(g, push_type, qbm, dt, bm: Beam, e2, b2, nthreads=1):
    lib().orc_beam_push(C.byref(g), push_type, qbm, dt, bm.n, ptr(bm.x), ptr(bm.y), ptr(bm.z),
                        ptr(bm.px), ptr(bm.py), ptr(bm.pz), ptr(e2), ptr(b2), nthreads)


def beam_update_bound(g, bm: Beam) -> int:
    return int(lib().orc_beam_update_bound(C.byref(g), bm.n, ptr(bm.x), ptr(bm.y), ptr(bm.z),
                                           ptr(bm.px), ptr(bm.py), ptr(bm.pz), ptr(bm.q)))


def load_plasma(g, seed, ppc1, ppc2, num_theta, qm=-1.0, density=1.0, uth=(0.0, 0.0, 0.0)) -> Plasma:
    n = g.nr * ppc1 * ppc2 * num_theta
    pl = Plasma(n)
    r = Rng()
    lib().orc_rng_seed(C.byref(r), seed)
    u = np.array(uth, np.float64)
    n = lib().orc_load_plasma(C.byref(g), C.byref(r), ppc1, ppc2, num_theta, qm, density, ptr(u),
                              ptr(pl.x), ptr(pl.y), ptr(pl.px), ptr(pl.py), ptr(pl.pz),
                              ptr(pl.gamma), ptr(pl.psi), ptr(pl.q))
    return pl.trim(int(n))


def load_beam(g, seed, tot_num, tot_charge, qm, gamma, center, sigma, range_lo, range_hi,
              uth=(0.0, 0.0, 0.0), quiet=False, rng=None) -> Beam:
    d = BeamDesc(tot_num, tot_charge, qm, gamma, (C.c_double * 3)(*center), (C.c_double * 3)(*sigma),
                 (C.c_double * 3)(*range_lo), (C.c_double * 3)(*range_hi), (C.c_double * 3)(*uth),
                 int(quiet))
    bm = Beam(tot_num * (2 if quiet else 1))
    r = rng if rng is not None else Rng()
    if rng is None:
        lib().orc_rng_seed(C.byref(r), seed)
    n = lib().orc_load_beam(C.byref(g), C.byref(r), C.byref(d), ptr(bm.x), ptr(bm.y), ptr(bm.z),
                            ptr(bm.px), ptr(bm.py), ptr(bm.pz), ptr(bm.q))
    return bm.trim(int(n))


class Sim:
    """One-species, N-beam driver around orc_sim_run_3dstep (simulation_class.f03:294-512)."""

    def __init__(self, g: Grid, *, iter_max=50, iter_reltol=1e-6, iter_abstol=0.0, dt3d=10.0,
                 sp_qbm=-1.0, sp_push_type=PUSH_ROBUST, neutralized=True, sp_npmax=1,
                 beams=(), nthreads=1, smooth_order=0, extrap=0, neutral=None, lasers=(), sp_ppc_r=2):
        d = SimDesc()
        d.g = g
        d.iter_max, d.iter_reltol, d.iter_abstol, d.dt3d = iter_max, iter_reltol, iter_abstol, dt3d
        d.sp_qbm, d.sp_push_type, d.sp_neutralized, d.sp_npmax = sp_qbm, sp_push_type, int(neutralized), sp_npmax
        d.nbeams = len(beams)
        for k, (qbm, ptype, npmax) in enumerate(beams):
            d.beam_qbm[k], d.beam_push_type[k], d.beam_npmax[k] = qbm, ptype, max(1, npmax)
        d.nthreads = nthreads
        d.smooth_order = smooth_order
        d.extrap = extrap
        self.neutral = neutral
        if neutral:
            # neutral: dict(adk=[(p1, p2, p3), ...], wp, density, ppc=(a, b), num_theta, qm, qbm,
            #               push_type, npmax)
            d.neut_levels = len(neutral["adk"])
            for i, (a, b_, c) in enumerate(neutral["adk"]):
                d.neut_adk[3 * i], d.neut_adk[3 * i + 1], d.neut_adk[3 * i + 2] = a, b_, c
            d.neut_wp, d.neut_density = neutral["wp"], neutral["density"]
            d.neut_ppc1, d.neut_ppc2 = neutral["ppc"]
            d.neut_num_theta = neutral["num_theta"]
            d.neut_qm, d.neut_qbm = neutral.get("qm", -1.0), neutral.get("qbm", -1.0)
            d.neut_push_type = neutral.get("push_type", PUSH_ROBUST)
            d.neut_npmax = neutral["npmax"]
        # lasers: [dict(k0=, iter=, ar=[nz][P][nr], ai=[nz][P][nr])]; nr a power of two
        d.nlasers = len(lasers)
        for k, ls in enumerate(lasers):
            d.laser_k0[k], d.laser_iter[k] = ls["k0"], ls["iter"]
        d.sp_ppc_r = sp_ppc_r
        self.g = g
        self.nlasers = len(lasers)
        self.h = lib().orc_sim_create(C.byref(d))
        for k, ls in enumerate(lasers):
            ar = np.ascontiguousarray(ls["ar"], np.float64)
            ai = np.ascontiguousarray(ls["ai"], np.float64)
            lib().orc_sim_set_laser(self.h, k, ptr(ar), ptr(ai))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sim_destroy(self.h)
            self.h = None

    def set_plasma(self, pl: Plasma):
        lib().orc_sim_set_plasma(self.h, pl.n, ptr(pl.x), ptr(pl.y), ptr(pl.px), ptr(pl.py),
                                 ptr(pl.pz), ptr(pl.gamma), ptr(pl.psi), ptr(pl.q))

    def set_beam(self, k, bm: Beam):
        lib().orc_sim_set_beam(self.h, k, bm.n, ptr(bm.x), ptr(bm.y), ptr(bm.z), ptr(bm.px),
                               ptr(bm.py), ptr(bm.pz), ptr(bm.q))

    def run_3dstep(self, push_beams=True):
        iters = (C.c_int * self.g.nz)()
        rel = np.zeros(self.g.nz)
        lib().orc_sim_run_3dstep(self.h, int(push_beams), iters, ptr(rel))
        return np.array(iters[:], dtype=np.int32), rel

    def begin_3dstep(self):
        lib().orc_sim_begin_3dstep(self.h)

    def slice(self, j):
        it, rel = C.c_int(), C.c_double()
        lib().orc_sim_slice(self.h, j, C.byref(it), C.byref(rel))
        return it.value, rel.value

    def end_3dstep(self, push_beams=True):
        lib().orc_sim_end_3dstep(self.h, int(push_beams))

    def field(self, name):
        nc = C.c_int()
        p = lib().orc_sim_field(self.h, name.encode(), C.byref(nc))
        P = 2 * self.g.max_mode + 1
        return np.ctypeslib.as_array(p, shape=(P, nc.value, self.g.nr + 2)).copy()

    def store(self, name):
        nc = C.c_int()
        p = lib().orc_sim_store(self.h, name.encode(), C.byref(nc))
        P = 2 * self.g.max_mode + 1
        return np.ctypeslib.as_array(p, shape=(self.g.nz + 1, P, nc.value, self.g.nr + 2)).copy()

    def plasma(self) -> Plasma:
        ps = [D() for _ in range(8)]
        n = int(lib().orc_sim_plasma(self.h, *[C.byref(p) for p in ps]))
        pl = Plasma(n)
        for k, p in zip(Plasma.NAMES, ps):
            setattr(pl, k, np.ctypeslib.as_array(p, shape=(max(n, 1),))[:n].copy())
        return pl

    def neutral_plasma(self) -> Plasma:
        """The neutral gas's ionised electrons."""
        ps = [D() for _ in range(8)]
        n = int(lib().orc_sim_neutral(self.h, *[C.byref(p) for p in ps]))
        pl = Plasma(n)
        for k, p in zip(Plasma.NAMES, ps):
            setattr(pl, k, np.ctypeslib.as_array(p, shape=(max(n, 1),))[:n].copy())
        return pl

    def laser(self, k):
        """Laser k's envelope (a_r, a_i) over slices 1..nz: [nz][P][nr + 2] each."""
        pr, pi = D(), D()
        lib().orc_sim_laser(self.h, k, C.byref(pr), C.byref(pi))
        P = 2 * self.g.max_mode + 1
        shape = (self.g.nz + 3, P, self.g.nr + 2)
        return tuple(np.ctypeslib.as_array(p, shape=shape)[2:self.g.nz + 2].copy() for p in (pr, pi))

    def multi_ion(self) -> np.ndarray:
        """Ionisation state [n_theta][nr][levels + 2] (levels, neutral fraction, quantised mean)."""
        L = len(self.neutral["adk"])
        p = lib().orc_sim_multi_ion(self.h)
        return np.ctypeslib.as_array(p, shape=(self.neutral["num_theta"], self.g.nr, L + 2)).copy()

    def beam(self, k) -> Beam:
        ps = [D() for _ in range(7)]
        n = int(lib().orc_sim_beam(self.h, k, *[C.byref(p) for p in ps]))
        bm = Beam(n)
        for kk, p in zip(Beam.NAMES, ps):
            setattr(bm, kk, np.ctypeslib.as_array(p, shape=(max(n, 1),))[:n].copy())
        return bm
