"""Python mirror of the reference's type-bound call surface over the C ABI.

The names follow QPAD's Fortran classes so that a test or driver written against the
reference reads the same way here:

    Simulation        simulation + sim_fields + options        (simulation_class.f03, sim_fields_class.f03)
    Field             one sim_fields object (psi, e, e_spe, b, ...) with its solve/copy_slice
    Species2D         species2d: qdp, amjdp, push_u, push_x, interp_psi, sort, renew
    Beam3D            beam3d: qdp, push

Array layouts on the Python side:
    slice field    float64 (P, ncomp, nr + 2)    P = 2M+1 parts (0: m=0, 2m-1: Re m, 2m: Im m)
    particles      x (np, 2) / (nb, 3), p (n, 3) C-ordered, i.e. the Fortran x(2,np), p(3,np)
Errors raise QpadError with the library's message; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as K


class QpadError(RuntimeError):
    pass


def _dp(a: np.ndarray):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, "float64 C-contiguous array expected"
    return a.ctypes.data_as(K.D)


class Field:
    """One field object of sim_fields (source/sim_fields_class.f03:45-89)."""

    def __init__(self, sim: "Simulation", name: str):
        self.sim, self.name, self.id = sim, name, K.FIELD_ID[name]
        self.ncomp = K.FIELD_NCOMP[name]

    # ufield f1 mirror
    def upload(self, arr: np.ndarray):
        s = self.sim
        arr = np.asarray(arr, dtype=np.float64)
        assert arr.shape == (s.P, self.ncomp, s.nr + 2)
        for p in range(s.P):
            s._check(s.lib.qpad_field_upload(s.h, self.id, p, _dp(np.ascontiguousarray(arr[p].T))))

    def download(self) -> np.ndarray:
        s = self.sim
        out = np.zeros((s.P, self.ncomp, s.nr + 2))
        buf = np.zeros((s.nr + 2, self.ncomp))
        for p in range(s.P):
            s._check(s.lib.qpad_field_download(s.h, self.id, p, _dp(buf)))
            out[p] = buf.T
        return out

    def store(self, slice_: int) -> np.ndarray:
        """f2(:, :, slice) of the 3D store, slice 1..nz+1."""
        s = self.sim
        out = np.zeros((s.P, self.ncomp, s.nr + 2))
        buf = np.zeros((s.nr + 2, self.ncomp))
        for p in range(s.P):
            s._check(s.lib.qpad_store_download(s.h, self.id, slice_, p, _dp(buf)))
            out[p] = buf.T
        return out

    def store_all(self, lo: int = 1, n: int | None = None) -> np.ndarray:
        """Slices lo .. lo+n-1 of the 3D store (default: 1..nz) in one copy, shaped
        (n, P, ncomp, nr + 2)."""
        s = self.sim
        n = s.nz - lo + 1 if n is None else n
        out = np.empty((n, s.P, self.ncomp, s.nr + 2))
        s._check(s.lib.qpad_store_read(s.h, self.id, lo, n, _dp(out)))
        return out

    def store_upload(self, slice_: int, arr: np.ndarray):
        s = self.sim
        arr = np.asarray(arr, dtype=np.float64)
        for p in range(s.P):
            s._check(s.lib.qpad_store_upload(s.h, self.id, slice_, p, _dp(np.ascontiguousarray(arr[p].T))))

    def fill(self, v: float):
        self.sim._check(self.sim.lib.qpad_field_fill(self.sim.h, self.id, float(v)))

    def store_fill(self, v: float):
        self.sim._check(self.sim.lib.qpad_store_fill(self.sim.h, self.id, float(v)))

    def scale(self, v: float):
        self.sim._check(self.sim.lib.qpad_field_scale(self.sim.h, self.id, float(v)))

    def copy_slice(self, j: int, direction: int):
        self.sim._check(self.sim.lib.qpad_field_copy_slice(self.sim.h, self.id, j, direction))

    def solve(self, *srcs: "Field"):
        """The reference's generic `solve`, dispatched on this field and the sources."""
        s, L = self.sim, self.sim.lib
        n = self.name
        if n == "psi" and len(srcs) == 1:
            r = L.qpad_solve_psi(s.h, self.id, srcs[0].id)
        elif n in ("e", "e_spe") and len(srcs) == 1:
            r = L.qpad_solve_ez(s.h, self.id, srcs[0].id)
        elif n in ("e", "e_spe") and len(srcs) == 2:
            r = L.qpad_solve_et(s.h, self.id, srcs[0].id, srcs[1].id)
        elif n in ("b", "b_spe", "b_beam") and len(srcs) == 1 and srcs[0].ncomp == 1:
            r = L.qpad_solve_bt_beam(s.h, self.id, srcs[0].id)
        elif n in ("b", "b_spe", "b_beam") and len(srcs) == 1:
            r = L.qpad_solve_bz(s.h, self.id, srcs[0].id)
        elif n in ("b", "b_spe", "b_beam") and len(srcs) == 2:
            r = L.qpad_solve_bt_iter(s.h, self.id, srcs[0].id, srcs[1].id)
        elif n == "dcu" and len(srcs) == 2:
            r = L.qpad_solve_djdxi(s.h, self.id, srcs[0].id, srcs[1].id)
        else:
            raise QpadError(f"no solve for {n} with {[x.name for x in srcs]}")
        s._check(r)


def add_f1(a: Field, b: Field, c: Field):
    """c = a + b (add_f1_binary)."""
    a.sim._check(a.sim.lib.qpad_field_add(a.sim.h, a.id, b.id, c.id))


def add_f1_dim(a: Field, b: Field, adim, bdim):
    """b(bdim,:) += a(adim,:) (add_f1_unitary_dim), 1-based components."""
    ad = np.asarray(adim, np.int32)
    bd = np.asarray(bdim, np.int32)
    a.sim._check(a.sim.lib.qpad_field_add_dim(a.sim.h, a.id, b.id, ad.ctypes.data_as(K.I32P),
                                              bd.ctypes.data_as(K.I32P), len(ad)))


@dataclass
class SliceStats:
    iters: int
    rel_res: float
    abs_res: float


class Laser:
    """A laser envelope on the device (advanced by every 3D step)."""

    def __init__(self, sim, h):
        self.sim, self.h = sim, h

    def download(self):
        """(a_r, a_i), each [nz][P][nr + 2] over slices 1..nz."""
        s = self.sim
        ar = np.zeros((s.nz, s.P, s.nr + 2))
        ai = np.zeros((s.nz, s.P, s.nr + 2))
        s._check(s.lib.qpad_laser_download(self.h, _dp(ar), _dp(ai)))
        return ar, ai


class Simulation:
    """Context: grid + field set + species + beams on one GPU (one CUDA stream)."""

    def __init__(self, nr, nz, max_mode, dr, dxi, *, bnd=K.BND_OPEN, relax_fac=None, iter_max=50,
                 iter_reltol=1e-6, iter_abstol=0.0, dt=10.0, precision=K.PREC_FP64, device=0):
        self.lib = K.load()
        d = K.GridDesc(nr, nz, max_mode, bnd, dr, dxi, -1.0 if relax_fac is None else relax_fac, iter_max,
                       iter_reltol, iter_abstol, dt, precision, device)
        h = C.c_void_p()
        r = self.lib.qpad_ctx_create(C.byref(d), C.byref(h))
        if r != 0:
            raise QpadError(f"qpad_ctx_create failed ({r}): {self.lib.qpad_last_error(None).decode()}")
        self.h = h
        self.nr, self.nz, self.max_mode, self.P = nr, nz, max_mode, 2 * max_mode + 1
        self.dr, self.dxi, self.dt = dr, dxi, dt
        self.iter_max = iter_max
        self.fields = {n: Field(self, n) for n in K.FIELDS}
        self.species: list[Species2D] = []
        self.beams: list[Beam3D] = []
        self.lasers: list[Laser] = []

    def __getattr__(self, name):
        f = self.__dict__.get("fields")
        if f is not None and name in f:
            return f[name]
        raise AttributeError(name)

    def _check(self, r):
        if r != 0:
            raise QpadError(f"qpad error {r}: {self.lib.qpad_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            for s in list(self.species):
                s.h = None
            for b in list(self.beams):
                b.h = None
            self.lib.qpad_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        self._check(self.lib.qpad_synchronize(self.h))

    def add_species(self, x, p, gamma, psi, q, *, qbm=-1.0, push_type=K.PUSH2_ROBUST, neutralized=True,
                    npmax=None, sort_freq=0, ppc_r=None) -> "Species2D":
        """A plasma species from particle arrays; push_type PUSH2_*_PGC makes it see the lasers,
        ppc_r (its radial particles per cell) sets the on-axis factor of its susceptibility."""
        sp = Species2D(self, x, p, gamma, psi, q, qbm=qbm, push_type=push_type, neutralized=neutralized,
                       npmax=npmax, sort_freq=sort_freq)
        self.species.append(sp)
        if ppc_r is not None:
            self._check(self.lib.qpad_species_set_radial_ppc(sp.h, int(ppc_r)))
        return sp

    def add_laser(self, ar, ai, *, k0, iteration=1) -> "Laser":
        """A laser envelope (field_laser_class.f03) from its initial a_r, a_i [nz][P][nr]
        (qpad_gb300.lasers.launch evaluates the reference's profiles)."""
        ar = np.ascontiguousarray(ar, np.float64).reshape(self.nz, self.P, self.nr)
        ai = np.ascontiguousarray(ai, np.float64).reshape(self.nz, self.P, self.nr)
        d = K.LaserDesc(float(k0), int(iteration))
        h = C.c_void_p()
        self._check(self.lib.qpad_laser_create(self.h, C.byref(d), _dp(ar), _dp(ai), C.byref(h)))
        lz = Laser(self, h)
        self.lasers.append(lz)
        return lz

    def chi_store(self) -> np.ndarray:
        """The plasma susceptibility of the last 3D step, [nz][P][nr + 2]."""
        out = np.zeros((self.nz, self.P, self.nr + 2))
        self._check(self.lib.qpad_laser_chi_download(self.h, _dp(out)))
        return out

    def add_neutral(self, adk, *, wp, density, ppc=(2, 1), num_theta=8, qm=-1.0, qbm=-1.0,
                    push_type=K.PUSH2_ROBUST, npmax=None) -> "Species2D":
        """An ionising neutral gas (neutral_class.f03): `adk` = [(p1, p2, p3)] per ionisation
        level (see qpad_gb300.neutrals), wp the plasma frequency of n0 in 1/s, density in n0.
        Its electrons appear during each 3D step; npmax bounds them (default: every level of
        every cell ionised)."""
        import numpy as np
        a = np.ascontiguousarray(np.asarray(adk, np.float64).reshape(-1, 3))
        levels = len(a)
        if npmax is None:
            npmax = self.nr * ppc[0] * ppc[1] * num_theta * levels + 1024
        d = K.NeutralDesc(qm, qbm, push_type, levels, a.ctypes.data_as(K.D), wp, density, ppc[0], ppc[1],
                          num_theta, int(npmax))
        h = C.c_void_p()
        self._check(self.lib.qpad_neutral_create(self.h, C.byref(d), C.byref(h)))
        sp = Species2D.__new__(Species2D)
        sp.sim, sp.h, sp.npmax, sp.qbm, sp.push_type = self, h, int(npmax), qbm, push_type
        sp.levels, sp.num_theta = levels, num_theta
        self.species.append(sp)
        return sp

    def add_beam(self, x, p, q, *, qbm=-1.0, push_type=K.PUSH3_REDUCED, evolution=True, npmax=None) -> "Beam3D":
        bm = Beam3D(self, x, p, q, qbm=qbm, push_type=push_type, evolution=evolution, npmax=npmax)
        self.beams.append(bm)
        return bm

    def conv_test(self, b: Field, op: str, dim: int = 2):
        rel, ab = C.c_double(), C.c_double()
        self._check(self.lib.qpad_conv_test(self.h, b.id, dim, 0 if op == "record" else 1, C.byref(rel), C.byref(ab)))
        return rel.value, ab.value

    def use_graph(self, on: bool):
        """Run 3D steps as one CUDA graph (default) or drive slices/iterations from the host."""
        self._check(self.lib.qpad_set_graph(self.h, int(on)))

    def set_smooth(self, order: int):
        """Binomial smoothing passes (0 .. 64) of the species' charge and current deposits
        (the species' smooth_order)."""
        self._check(self.lib.qpad_set_smooth(self.h, int(order)))

    def set_guess_extrapolation(self, order: int, weight: float = 1.0):
        """Initial B-perp guess of every slice: 0 carries B-perp(j-1) as the reference does, 1
        and 2 extrapolate it linearly / quadratically from the previous slices; `weight` is
        the fraction of the extrapolation's change to the carried value that is applied."""
        self._check(self.lib.qpad_set_guess_extrapolation(self.h, int(order), float(weight)))

    def graph_active(self):
        """(whether the last 3D step ran as a graph, reason when it did not)."""
        a = C.c_int()
        self._check(self.lib.qpad_graph_active(self.h, C.byref(a)))
        return bool(a.value), self.lib.qpad_graph_status(self.h).decode()

    def launch_count(self) -> int:
        n = C.c_int64()
        self._check(self.lib.qpad_launch_count(self.h, C.byref(n)))
        return n.value

    def profile(self, on: bool):
        self._check(self.lib.qpad_profile_enable(self.h, int(on)))

    def profile_read(self, name: str):
        """(total device ms, launches) of one kernel family since profiling was enabled."""
        ms, n = C.c_double(), C.c_int64()
        self._check(self.lib.qpad_profile_read(self.h, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def slice_step(self, j: int) -> SliceStats:
        st = K.SliceStats()
        self._check(self.lib.qpad_slice_step(self.h, j, C.byref(st)))
        return SliceStats(st.iters, st.rel_res, st.abs_res)

    def run_3d_step(self, push_beams=True):
        """One 3D step; returns (iterations per slice, final rel_res per slice)."""
        st = (K.SliceStats * self.nz)()
        self._check(self.lib.qpad_3d_step(self.h, int(push_beams), st))
        return (np.array([s.iters for s in st], np.int32), np.array([s.rel_res for s in st]))

    def autotune(self, reps=20) -> dict:
        """Picks the fastest launch shapes of this simulation's kernels on this GPU."""
        r = K.TuneResult()
        self._check(self.lib.qpad_autotune(self.h, reps, C.byref(r)))
        return {"iter_cluster": r.iter_cluster, "iter_us": r.iter_us, "item_ppl": r.item_ppl,
                "deposit_us": r.deposit_us}

    def set_launch_shapes(self, iter_cluster=0, item_ppl=0):
        """Launch shapes by hand (0 keeps one): iteration CTAs per mode, deposit particles per lane."""
        self._check(self.lib.qpad_set_launch_shapes(self.h, int(iter_cluster), int(item_ppl)))

    def set_graph_unroll(self, iterations: int):
        """Predictor-corrector iterations per body of the step graph's iteration loop (1 .. 4)."""
        self._check(self.lib.qpad_set_graph_unroll(self.h, int(iterations)))


class Batch:
    """Independent simulations on one GPU advanced together: one 3D step of all of them is
    one CUDA graph launch of their slice loops (qpad_batch_step)."""

    def __init__(self, sims):
        self.sims = list(sims)
        self.lib = K.load()
        arr = (C.c_void_p * len(self.sims))(*[s.h.value for s in self.sims])
        h = C.c_void_p()
        r = self.lib.qpad_batch_create(arr, len(self.sims), C.byref(h))
        if r != 0:
            raise QpadError(f"qpad_batch_create failed ({r})")
        self.h = h

    def step(self, push_beams=True):
        """One 3D step of every simulation; returns the iterations per slice of each."""
        bufs = [(K.SliceStats * s.nz)() for s in self.sims]
        ptrs = (C.POINTER(K.SliceStats) * len(bufs))(*[C.cast(b, C.POINTER(K.SliceStats)) for b in bufs])
        r = self.lib.qpad_batch_step(self.h, int(push_beams), ptrs)
        if r != 0:
            raise QpadError(f"qpad_batch_step failed ({r}): {self.lib.qpad_batch_last_error(self.h).decode()}")
        return [np.array([s.iters for s in b], np.int32) for b in bufs]

    def autotune(self, reps=1) -> dict:
        """Times whole batch steps under each cluster policy of the iteration kernels and
        iterations per loop body, and keeps the fastest (qpad_batch_autotune)."""
        r = K.BatchTuneResult()
        e = self.lib.qpad_batch_autotune(self.h, int(reps), C.byref(r))
        if e != 0:
            raise QpadError(f"qpad_batch_autotune failed ({e}): {self.lib.qpad_batch_last_error(self.h).decode()}")
        return {"policy": "smallest cluster that fits" if r.policy == 0 else f"own shape capped at {r.policy} CTAs",
                "unroll": r.unroll, "step_ms": r.step_ms}

    def close(self):
        if getattr(self, "h", None):
            self.lib.qpad_batch_destroy(self.h)
            self.h = None


class Species2D:
    def __init__(self, sim: Simulation, x, p, gamma, psi, q, *, qbm, push_type, neutralized, npmax, sort_freq):
        self.sim = sim
        n = len(q)
        npmax = int(npmax or max(1, 2 * n))
        d = K.SpeciesDesc(qbm, push_type, int(neutralized), npmax, sort_freq)
        h = C.c_void_p()
        x, p, gamma, psi, q = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, p, gamma, psi, q))
        sim._check(sim.lib.qpad_species_create(sim.h, C.byref(d), _dp(x), _dp(p), _dp(gamma), _dp(psi), _dp(q), n,
                                               C.byref(h)))
        self.h, self.npmax, self.qbm, self.push_type = h, npmax, qbm, push_type

    def renew(self, x, p, gamma, psi, q):
        x, p, gamma, psi, q = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, p, gamma, psi, q))
        self.sim._check(self.sim.lib.qpad_species_renew(self.h, _dp(x), _dp(p), _dp(gamma), _dp(psi), _dp(q),
                                                        len(q)))

    def reset(self):
        """renew from the device copy of the last uploaded particles (no host traffic)."""
        self.sim._check(self.sim.lib.qpad_species_reset(self.h))

    def count(self) -> int:
        n = C.c_int64()
        self.sim._check(self.sim.lib.qpad_species_count(self.h, C.byref(n)))
        return n.value

    def download(self):
        n = self.count()
        x, p = np.zeros((max(n, 1), 2)), np.zeros((max(n, 1), 3))
        g, ps, q = np.zeros(max(n, 1)), np.zeros(max(n, 1)), np.zeros(max(n, 1))
        nn = C.c_int64()
        self.sim._check(self.sim.lib.qpad_species_download(self.h, _dp(x), _dp(p), _dp(g), _dp(ps), _dp(q),
                                                           C.byref(nn)))
        n = nn.value
        return x[:n], p[:n], g[:n], ps[:n], q[:n]

    def qdp(self, q: Field):
        self.sim._check(self.sim.lib.qpad_species_qdp(self.h, q.id))

    def cbq(self, pos: int, q: Field, cu: Field):
        """rho = (rho - Jz) + Jz into q, then q's slice `pos` into its 3D store (cbq_species2d)."""
        self.sim._check(self.sim.lib.qpad_species_cbq(self.h, q.id, cu.id, int(pos)))

    def amjdp(self, ef: Field, bf: Field, cu: Field, amu: Field, dcu: Field, dt: float):
        self.sim._check(self.sim.lib.qpad_species_amjdp(self.h, ef.id, bf.id, cu.id, amu.id, dcu.id, dt))

    def push_u(self, ef: Field, bf: Field, dt: float):
        self.sim._check(self.sim.lib.qpad_species_push_u(self.h, ef.id, bf.id, dt))

    def push_x(self, dt: float):
        self.sim._check(self.sim.lib.qpad_species_push_x(self.h, dt))

    def interp_psi(self, psi: Field):
        self.sim._check(self.sim.lib.qpad_species_interp_psi(self.h, psi.id))

    def sort(self):
        self.sim._check(self.sim.lib.qpad_species_sort(self.h))

    def ionisation_state(self):
        """A neutral gas's state [num_theta][nr][levels + 2]: the fractions in each level, the
        neutral fraction and the mean ionisation quantised to the particles per cell."""
        out = np.zeros((self.num_theta, self.sim.nr, self.levels + 2))
        self.sim._check(self.sim.lib.qpad_neutral_state_download(self.h, _dp(out)))
        return out


class Beam3D:
    def __init__(self, sim: Simulation, x, p, q, *, qbm, push_type, evolution, npmax):
        self.sim = sim
        n = len(q)
        npmax = int(npmax or max(1, n))
        d = K.BeamDesc(qbm, push_type, int(evolution), npmax)
        h = C.c_void_p()
        x, p, q = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, p, q))
        sim._check(sim.lib.qpad_beam_create(sim.h, C.byref(d), _dp(x), _dp(p), _dp(q), n, C.byref(h)))
        self.h = h
        self.qbm, self.push_type, self.evolution, self.npmax = qbm, push_type, bool(evolution), npmax

    def count(self) -> int:
        n = C.c_int64()
        self.sim._check(self.sim.lib.qpad_beam_count(self.h, C.byref(n)))
        return n.value

    def download(self):
        n = self.count()
        x, p, q = np.zeros((max(n, 1), 3)), np.zeros((max(n, 1), 3)), np.zeros(max(n, 1))
        nn = C.c_int64()
        self.sim._check(self.sim.lib.qpad_beam_download(self.h, _dp(x), _dp(p), _dp(q), C.byref(nn)))
        n = nn.value
        return x[:n], p[:n], q[:n]

    def qdp(self, q: Field):
        self.sim._check(self.sim.lib.qpad_beam_qdp(self.h, q.id))

    def push(self, ef: Field, bf: Field):
        self.sim._check(self.sim.lib.qpad_beam_push(self.h, ef.id, bf.id))


# ---- loaders --------------------------------------------------------------------------------
def load_plasma(nr, dr, seed, ppc1, ppc2, num_theta, qm=-1.0, density=1.0, uth=(0.0, 0.0, 0.0), rng=None):
    """fdist2d::inject for a uniform plasma; returns (x(np,2), p(np,3), gamma, psi, q)."""
    L = K.load()
    cap = nr * ppc1 * ppc2 * num_theta
    x, p = np.zeros((cap, 2)), np.zeros((cap, 3))
    g, ps, q = np.zeros(cap), np.zeros(cap), np.zeros(cap)
    r = rng if rng is not None else K.Rng()
    if rng is None:
        L.qpad_rng_seed(C.byref(r), seed)
    u = np.asarray(uth, np.float64)
    n = L.qpad_load_plasma(nr, dr, C.byref(r), ppc1, ppc2, num_theta, qm, density, _dp(u), _dp(x), _dp(p), _dp(g),
                           _dp(ps), _dp(q), cap)
    if n < 0:
        raise QpadError("qpad_load_plasma failed")
    return x[:n], p[:n], g[:n], ps[:n], q[:n]


def load_beam(nr, nz, dr, dxi, seed, tot_num, tot_charge, qm, gamma, center, sigma, range_lo, range_hi,
              uth=(0.0, 0.0, 0.0), quiet=False, rng=None):
    """fdist3d_rnd::inject with Gaussian profiles; returns (x(nb,3), p(nb,3), q)."""
    L = K.load()
    d = K.BeamLoadDesc(tot_num, tot_charge, qm, gamma, (C.c_double * 3)(*center), (C.c_double * 3)(*sigma),
                       (C.c_double * 3)(*range_lo), (C.c_double * 3)(*range_hi), (C.c_double * 3)(*uth), int(quiet))
    cap = tot_num * (2 if quiet else 1)
    x, p, q = np.zeros((max(cap, 1), 3)), np.zeros((max(cap, 1), 3)), np.zeros(max(cap, 1))
    r = rng if rng is not None else K.Rng()
    if rng is None:
        L.qpad_rng_seed(C.byref(r), seed)
    n = L.qpad_load_beam(nr, nz, dr, dxi, C.byref(r), C.byref(d), _dp(x), _dp(p), _dp(q), cap)
    if n < 0:
        raise QpadError("qpad_load_beam failed")
    return x[:n], p[:n], q[:n]
