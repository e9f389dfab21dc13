"""Reads the reference's JSON input deck and builds the simulation it describes.

The deck is the reference's own input file (json-fortran dialect: ``!`` starts a comment
outside strings).  Keys follow the reference's readers:

* ``simulation``: grid, box, max_mode, dt, time (3D steps = time / dt,
  simulation_class.f03:144-147), iter_max / iter_reltol / iter_abstol (:158-160),
  random_seed (:125), field_boundary and relax_fac (sim_fields_class.f03:116, 137-140),
  nbeams / nspecies / nneutrals / nlasers (:161-164), interpolation (sim_plasma_class.f03:87),
  read_restart / restart_timestep (:150-152).
* ``species(i)`` (fdist2d_class.f03:142-265, sim_plasma_class.f03:119-142): profile, ppc,
  num_theta, q, m, density, uth, neutralized, sort_freq, npmax, push_type, smooth_order.
* ``beam(i)`` with ``profile_type`` "random" (beam3d_class.f03:85-111,
  fdist3d_rnd_class.f03:120-290): profile, total_num, total_charge, q, m, gamma, range1-3,
  gauss_center, gauss_sigma, uth, geometry, evolution, quiet_start, push_type.

Only what this library simulates is accepted: a box starting at r = 0 and z = 0, uniform
plasma species, Gaussian random-profile beams in cartesian geometry without spin, linear
interpolation, no lasers and no neutrals.  Anything else raises NotImplementedError naming
the key, rather than being simulated differently.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field

from . import _capi as K
from .api import Simulation, load_beam, load_plasma


def strip_comments(text: str) -> str:
    """Removes json-fortran ``!`` comments (to the end of the line, outside strings)."""
    out, in_str, esc, skip = [], False, False, False
    for ch in text:
        if skip:
            if ch == "\n":
                skip = False
                out.append(ch)
            continue
        if in_str:
            out.append(ch)
            if esc:
                esc = False
            elif ch == "\\":
                esc = True
            elif ch == '"':
                in_str = False
            continue
        if ch == '"':
            in_str = True
        elif ch == "!":
            skip = True
            continue
        out.append(ch)
    return "".join(out)


@dataclass
class InputDeck:
    nr: int
    nz: int
    dr: float
    dxi: float
    max_mode: int
    dt: float
    n_steps: int
    iter_max: int
    iter_reltol: float
    iter_abstol: float
    bnd: int
    relax_fac: float | None
    seed: int
    species: list = field(default_factory=list)   # dicts: loader and species arguments
    beams: list = field(default_factory=list)     # dicts: loader and beam arguments
    start_step: int = 1                           # first 3D step (restart_timestep + 1 on a restart)
    read_restart: bool = False


def _need(sect: dict, key: str, where: str):
    if key not in sect:
        raise ValueError(f"{where}.{key} is missing")
    return sect[key]


def _unsupported(cond: bool, what: str):
    if cond:
        raise NotImplementedError(what)


def parse(text_or_dict) -> InputDeck:
    """An InputDeck from the deck's text (or an already-loaded dict)."""
    d = json.loads(strip_comments(text_or_dict)) if isinstance(text_or_dict, str) else text_or_dict
    sim = _need(d, "simulation", "deck")
    nr, nz = (int(v) for v in _need(sim, "grid", "simulation"))
    box = _need(sim, "box", "simulation")
    r0, r1 = (float(v) for v in _need(box, "r", "simulation.box"))
    z0, z1 = (float(v) for v in _need(box, "z", "simulation.box"))
    _unsupported(r0 != 0.0 or z0 != 0.0, "simulation.box: only boxes starting at r = 0 and z = 0")
    _unsupported(int(sim.get("nlasers", 0)) != 0, "simulation.nlasers: lasers (PGC) are not built")
    _unsupported(int(sim.get("nneutrals", 0)) != 0, "simulation.nneutrals: neutrals / ionisation are not built")
    _unsupported(sim.get("interpolation", "linear") != "linear", "simulation.interpolation: only linear")
    alg = sim.get("algorithm", "standard")
    _unsupported(alg != "standard", f"simulation.algorithm: only the standard quasi-static loop ({alg})")
    fb = sim.get("field_boundary", "open")
    _unsupported(fb not in ("open", "zero"), f"simulation.field_boundary: {fb}")
    dt = float(_need(sim, "dt", "simulation"))
    time = float(_need(sim, "time", "simulation"))
    read_rst = bool(sim.get("read_restart", False))
    deck = InputDeck(
        nr=nr, nz=nz, dr=(r1 - r0) / nr, dxi=(z1 - z0) / nz, max_mode=int(_need(sim, "max_mode", "simulation")),
        dt=dt, n_steps=int(time / dt), iter_max=int(_need(sim, "iter_max", "simulation")),
        iter_reltol=float(_need(sim, "iter_reltol", "simulation")),
        iter_abstol=float(_need(sim, "iter_abstol", "simulation")),
        bnd=K.BND_OPEN if fb == "open" else K.BND_ZERO,
        relax_fac=float(sim["relax_fac"]) if "relax_fac" in sim else None,
        seed=int(sim.get("random_seed", 0)), read_restart=read_rst,
        start_step=int(sim.get("restart_timestep", 0)) + 1 if read_rst else 1)
    nspecies = int(sim.get("nspecies", len(d.get("species", []))))
    for i, s in enumerate(d.get("species", [])[:nspecies], start=1):
        w = f"species({i})"
        prof = list(s.get("profile", ["uniform", "uniform"]))
        _unsupported(prof != ["uniform", "uniform"], f"{w}.profile: only uniform plasma ({prof})")
        pt = s.get("push_type", "robust")
        _unsupported(pt not in ("robust", "standard"), f"{w}.push_type: {pt}")
        ppc = [int(v) for v in _need(s, "ppc", w)]
        q, m = float(_need(s, "q", w)), float(s.get("m", 1.0))
        uth = [float(v) for v in s.get("uth", [0.0, 0.0, 0.0])]
        deck.species.append(dict(
            ppc=(ppc[0], ppc[1]), num_theta=int(_need(s, "num_theta", w)), q=q, qbm=q / m,
            density=float(_need(s, "density", w)), uth=tuple(uth),
            push_type=K.PUSH2_ROBUST if pt == "robust" else K.PUSH2_STD,
            neutralized=bool(s.get("neutralized", True)), sort_freq=int(s.get("sort_freq", 0)),
            npmax=int(s["npmax"]) if "npmax" in s else None, smooth_order=int(s.get("smooth_order", 0))))
    nbeams = int(sim.get("nbeams", len(d.get("beam", []))))
    for i, b in enumerate(d.get("beam", [])[:nbeams], start=1):
        w = f"beam({i})"
        ptype = b.get("profile_type", "standard")
        _unsupported(ptype != "random", f"{w}.profile_type: only 'random' beams are built ({ptype})")
        prof = list(_need(b, "profile", w))
        _unsupported(prof != ["gaussian"] * 3, f"{w}.profile: only gaussian in all three directions ({prof})")
        _unsupported(b.get("geometry", "cartesian") != "cartesian", f"{w}.geometry: only cartesian")
        _unsupported(bool(b.get("has_spin", False)), f"{w}.has_spin: spin is not built")
        # beam-shaping keys of fdist3d_rnd (fdist3d_rnd_class.f03:286-314): the Twiss alpha
        # correlation and the xi-dependent transverse offsets
        for key in ("alpha", "perp_offset_x", "perp_offset_y"):
            _unsupported(key in b, f"{w}.{key}: not built")
        pt = b.get("push_type", "reduced")
        _unsupported(pt not in ("reduced", "boris"), f"{w}.push_type: {pt}")
        q, m = float(_need(b, "q", w)), float(b.get("m", 1.0))
        rng = [[float(v) for v in _need(b, f"range{k}", w)] for k in (1, 2, 3)]
        deck.beams.append(dict(
            tot_num=int(_need(b, "total_num", w)), tot_charge=float(_need(b, "total_charge", w)), qm=q,
            qbm=q / m, gamma=float(_need(b, "gamma", w)),
            center=tuple(float(v) for v in _need(b, "gauss_center", w)),
            sigma=tuple(float(v) for v in _need(b, "gauss_sigma", w)),
            range_lo=tuple(r[0] for r in rng), range_hi=tuple(r[1] for r in rng),
            uth=tuple(float(v) for v in b.get("uth", [0.0, 0.0, 0.0])), quiet=bool(b.get("quiet_start", False)),
            push_type=K.PUSH3_REDUCED if pt == "reduced" else K.PUSH3_BORIS, evolution=bool(b.get("evolution", True))))
    return deck


def read(path: str) -> InputDeck:
    with open(path) as f:
        return parse(f.read())


def stream_seed(seed: int, kind: int, k: int, step: int = 0) -> int:
    """Loader seed of one particle stream: species k (kind 0) at 3D step `step`, or beam k
    (kind 1), mixed from the tuple by numpy's SeedSequence, so that no two streams of a run
    coincide however many steps or species it has.  (The reference's random_seed 0 asks for
    an OS-chosen seed; here every seed, 0 included, is reproducible.)"""
    import numpy as np
    return int(np.random.SeedSequence([int(seed), int(kind), int(k), int(step)]).generate_state(1, np.uint64)[0])


def inputs(deck: InputDeck, step: int = 1, beams: bool = True):
    """Host arrays of every species (for 3D step `step`) and, with `beams`, every beam, from
    the deck's seed (one stream per species and step, one per beam: stream_seed)."""
    sp = []
    for k, s in enumerate(deck.species):
        sp.append(load_plasma(deck.nr, deck.dr, stream_seed(deck.seed, 0, k, step), s["ppc"][0], s["ppc"][1],
                              s["num_theta"], qm=s["q"], density=s["density"], uth=s["uth"]))
    bm = []
    for k, b in enumerate(deck.beams if beams else []):
        bm.append(load_beam(deck.nr, deck.nz, deck.dr, deck.dxi, stream_seed(deck.seed, 1, k), b["tot_num"],
                            b["tot_charge"], b["qm"], b["gamma"], b["center"], b["sigma"], b["range_lo"],
                            b["range_hi"], uth=b["uth"], quiet=b["quiet"]))
    return sp, bm


def build(deck: InputDeck, precision=K.PREC_FP64, device=0, restart_root: str = ".") -> Simulation:
    """The simulation the deck describes, with its species and beams on the device.  With
    read_restart the beams come from their restart files at restart_timestep under
    `restart_root` (sim_beams_class.f03:121-128) instead of the loader."""
    sim = Simulation(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi, bnd=deck.bnd, relax_fac=deck.relax_fac,
                     iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, iter_abstol=deck.iter_abstol, dt=deck.dt,
                     precision=precision, device=device)
    orders = {s["smooth_order"] for s in deck.species}
    _unsupported(len(orders) > 1, "species smooth_order: one order for all species")
    if orders and max(orders) > 0:
        sim.set_smooth(max(orders))
    sp, bm = inputs(deck, deck.start_step, beams=not deck.read_restart)
    for s, (x, p, g, ps, q) in zip(deck.species, sp):
        sim.add_species(x, p, g, ps, q, qbm=s["qbm"], push_type=s["push_type"], neutralized=s["neutralized"],
                        npmax=s["npmax"] or max(1, len(q)), sort_freq=s["sort_freq"])
    if deck.read_restart:
        from . import restart
        # the particles come from the files, the beam's parameters from the deck
        # (sim_beams_class.f03 reads only x, p and q back)
        restart.load_beams(sim, restart_root, deck.start_step - 1, len(deck.beams),
                           params=[dict(qbm=b["qbm"], push_type=b["push_type"], evolution=b["evolution"])
                                   for b in deck.beams])
        return sim
    for b, (x, p, q) in zip(deck.beams, bm):
        sim.add_beam(x, p, q, qbm=b["qbm"], push_type=b["push_type"], evolution=b["evolution"],
                     npmax=max(1, len(q)))
    return sim


def run(deck: InputDeck, sim: Simulation, steps: int | None = None):
    """Runs the deck's 3D steps start_step .. n_steps (the reference's `do i = start3d,
    nstep3d`, simulation_class.f03:294; none when a restart is already past the end), or
    `steps` steps from start_step: before every step after the first, each species is renewed
    from that step's loader stream, as the reference re-injects its plasma after each 3D step
    (species2d::renew, species2d_class.f03:154-184).  Returns the per-step (iterations per
    slice, rel_res)."""
    n = max(0, deck.n_steps - deck.start_step + 1) if steps is None else steps
    out = []
    for k in range(n):
        step = deck.start_step + k
        if k > 0:
            sp, _ = inputs(deck, step) if deck.species else ([], [])
            for spec, (x, p, g, ps, q) in zip(sim.species, sp):
                spec.renew(x, p, g, ps, q)
        out.append(sim.run_3d_step())
    return out
