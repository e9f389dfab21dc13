"""Benchmark of the quasi-static slice loop (one JSON line on rank 0).

A step is one 3D step of the c5 deck (the largest single-GPU shape: M=4, nr=2048, 4096
slices, 1.05e6 plasma particles per slice, 1e8 beam particles): beam charge deposit, every
slice with the full B-perp predictor-corrector (iter_reltol 1e-6), beam push, and the
plasma renewal that the reference performs after every 3D step.  The metric's first half,
plasma particle-pushes/s, is the headline value (one plasma particle advanced through one
slice, all of its predictor-corrector deposits included); B-perp iterations per slice are
reported beside it.  The headline path is the mixed-precision one (FP32 particles, FP64
solves); each slice's B-perp iteration starts from the linear extrapolation of the two
previous slices' converged B-perp (--guess-order 1, not in the reference, which carries
slice j-1's: --guess-order 0).  The plain FP64 path, with the carried guess, runs on the
same deck and inputs as the comparison arm
("compare", "speedup_vs_fp64", "iters_change_vs_fp64"), and the per-mode field error of
the mixed path against it over one whole 3D step from identical inputs is "max_mode_err"
(the FP64 path itself matches the FP64 oracle to 1e-9; the oracle is too slow for a whole
c5 step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--deck c5|c2|c1|c3] [--precision mixed|fp64] [--no-compare]

--impl reference times the reference algorithm's CPU implementation (the project's C
restatement of it, OpenMP over particles, every host core) on a bounded sample of the
same deck, with inputs from the oracle's own loaders; the Fortran reference itself cannot
be built on these machines.  Multi-GPU runs are independent replicas (one simulation per
GPU, different seeds).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-pushes/s & B⊥ iters/slice: mixed+learned vs plain FP64 @1e-4 err"
UNIT = "particle-pushes/s"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def _deck(args):
    from qpad_gb300 import decks          # pure Python: the deck shapes, no library load
    d = decks.DECKS[args.deck]()
    tags = []
    if args.slices:
        # profiling runs: the same slice workload over fewer slices
        d.nz = args.slices
        tags.append(f"nz{args.slices}")
    if args.beam_frac:
        # profiling runs: fewer beam particles (a few GB on the device at most)
        for b in d.beams:
            b.num = max(1, int(b.num * args.beam_frac))
        tags.append(f"beam{args.beam_frac:g}")
    if tags:
        d.name = d.name + "_" + "_".join(tags)
    return d


def oracle_inputs(deck):
    """The deck's plasma and beams from the oracle's own loaders (orc_load_plasma /
    orc_load_beam: the same seeded streams as the product's loaders, which the CPU tests
    check bit for bit), so that the CPU arm never loads the product library."""
    from oracle import oracle as O
    g = O.grid(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi)
    pl = O.load_plasma(g, deck.seed * 1000, deck.ppc[0], deck.ppc[1], deck.num_theta,
                       uth=(deck.uth, deck.uth, deck.uth))
    beams = []
    for k, b in enumerate(deck.beams):
        a = b.load_args(deck.nz, deck.dxi)
        if a["range_lo"][2] >= a["range_hi"][2]:              # beam entirely behind a shortened box
            beams.append(O.Beam(0))
            continue
        beams.append(O.load_beam(g, deck.seed * 1000 + 999 + k, a["tot_num"], a["tot_charge"], a["qm"], a["gamma"],
                                 a["center"], a["sigma"], a["range_lo"], a["range_hi"], uth=a["uth"]))
    return g, pl, beams


class CpuSample:
    """The oracle (C restatement of the reference loop, OpenMP over particles and modes) set up
    once for a deck; run(n) times its first n slices with every plasma particle, the beam
    charge of the whole deck deposited before the clock starts."""

    def __init__(self, deck, nthreads=None):
        from oracle import oracle as O
        self.deck = deck
        self.nthreads = nthreads or os.cpu_count()
        g, self.pl, beams = oracle_inputs(deck)
        self.sim = O.Sim(g, iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, iter_abstol=deck.iter_abstol,
                         dt3d=deck.dt, sp_npmax=self.pl.n,
                         beams=[(spec.qm, O.PUSH3_REDUCED, b.n) for b, spec in zip(beams, deck.beams)],
                         nthreads=self.nthreads)
        for k, bm in enumerate(beams):
            self.sim.set_beam(k, bm)

    def run(self, nslices):
        import numpy as np
        self.sim.set_plasma(self.pl)
        self.sim.begin_3dstep()
        t0 = time.perf_counter()
        its = [self.sim.slice(j)[0] for j in range(1, nslices + 1)]
        t = time.perf_counter() - t0
        return {"value": self.pl.n * nslices / t, "seconds": t, "iters_per_slice": float(np.mean(its)),
                "cores": self.nthreads, "slices": nslices, "particles_per_slice": self.pl.n}

    def sample_text(self, nslices):
        return (f"first {nslices} of {self.deck.nz} slices of {self.deck.name}, all {self.pl.n} plasma particles, "
                f"full predictor-corrector, beam charge of the whole deck deposited before the clock, "
                f"OpenMP oracle, inputs from the oracle's loaders")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    deck = _deck(args)
    cs = CpuSample(deck)
    vals, info = [], None
    for k in range(args.warmup + args.steps):
        info = cs.run(args.cpu_slices)
        if k >= args.warmup:
            vals.append(info["value"])
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": deck.name, "sample_slices": info["slices"]},
            "iters_per_slice": info["iters_per_slice"],
            # the same work counted per predictor-corrector iteration (a plasma particle through
            # one iteration of one slice), which does not depend on how many iterations the
            # sampled slices take
            "iteration_pushes_per_s": v * info["iters_per_slice"],
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": info["cores"], "kind": "port",
                             "sample": cs.sample_text(info["slices"])},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _stores(sim, names):
    from qpad_gb300.diagnostics import ERROR_FIELDS
    return {n: sim.fields[n].store_all() for n in (names or ERROR_FIELDS)}


def _first_step_stores(args, deck, inputs, prec, local):
    """The error fields' 3D stores after one 3D step from `inputs` (untimed)."""
    import qpad_gb300 as Q
    sim = Q.build_simulation(deck, precision=prec, device=local, inputs=inputs)
    sim.use_graph(args.graph == "on")
    sim.run_3d_step()
    out = _stores(sim, None)
    sim.close()
    return out


def _measure(args, deck, inputs, prec, local, dist, steps, warmup, full=True, guess=False, keep_stores=False,
             order=0):
    """Times `steps` 3D steps of one simulation (after `warmup` untimed ones) on the library's
    stream with CUDA events; with `full`, also the end-to-end pass with host buffers and one
    host-driven step with per-kernel event timing.  With keep_stores, the 3D stores of the
    first step (from the deck's inputs) come back in out["stores"]."""
    import qpad_gb300 as Q
    from qpad_gb300.replicas import reduce_timing
    sim = Q.build_simulation(deck, precision=prec, device=local, inputs=inputs)
    sim.set_guess_extrapolation(order)
    sim.use_graph(args.graph == "on")
    tune = sim.autotune(reps=20) if not args.no_autotune else None
    if args.item_ppl:
        sim.set_launch_shapes(item_ppl=args.item_ppl)
        if tune is not None:
            tune["item_ppl"] = args.item_ppl
    if guess:
        from qpad_gb300 import learned as LR
        LR.attach(sim, *LR.load(LR.weights_path(deck.max_mode), deck.max_mode, device=local))
    sp = sim.species[0]
    npl = len(inputs[0][4])

    def barrier():
        if dist is not None:
            dist.barrier()

    stores, first_iters = None, None
    for k in range(warmup):
        sp.reset()
        it, _ = sim.run_3d_step()
        if k == 0:
            first_iters = it
            if keep_stores:
                stores = _stores(sim, None)
    barrier()
    sim.synchronize()
    sim.profile(True)
    l0 = sim.launch_count()
    iters_tot = 0
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(steps):
            sp.reset()
            it, _ = sim.run_3d_step()
            iters_tot += int(it.sum())
        sim.synchronize()
        wall = time.perf_counter() - t0
    launches = sim.launch_count() - l0
    step_ms, nstep = sim.profile_read("step")
    sim.profile(False)
    graph_on, graph_why = sim.graph_active()
    dev_s = step_ms / 1e3 if nstep else wall
    barrier()
    pushes_step = npl * deck.nz
    dev_s, total_pushes = reduce_timing(dev_s, float(pushes_step * steps), dist)
    out = {"tune": tune, "value": total_pushes / dev_s, "ms_per_step": dev_s * 1e3 / steps,
           "iters_per_slice": iters_tot / (steps * deck.nz), "wall_s": wall, "launches": launches,
           "graph": {"active": graph_on, "status": graph_why}, "clocks": clk.summary(), "dev_s": dev_s,
           "pushes_step": pushes_step, "stores": stores, "first_iters": first_iters}
    if full:
        # kernel timing pass (outside the timed region): one host-driven step with CUDA events
        # bracketing every launch of each kernel family on the library's stream
        sim.use_graph(False)
        sim.profile(True)
        sp.reset()
        sim.run_3d_step()
        out["kern"] = {k: sim.profile_read(k) for k in ("amjdp", "iterate", "push", "qdeposit", "slice_begin",
                                                         "iter_e", "slice_end", "conv", "beam_push",
                                                         "beam_qdeposit", "step")}
        sim.profile(False)
        sim.use_graph(args.graph == "on")
        # end to end through the C ABI with host buffers: renew from host arrays every step and
        # read the per-slice statistics back
        x, p, g, ps, q = inputs[0]
        h2d = sum(a.nbytes for a in (x, p, g, ps, q))
        d2h = 0
        e2e_steps = max(1, min(steps, args.e2e_steps))
        e2e_t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sp.renew(x, p, g, ps, q)
            it, _ = sim.run_3d_step()
            d2h += deck.nz * 24
        e2e_s = time.perf_counter() - e2e_t0
        world = dist.get_world_size() if dist is not None else 1
        out["e2e"] = {"value": world * pushes_step * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps,
                      "timing": "host wall clock around qpad_species_renew + qpad_3d_step"}
    sim.close()
    return out


def run_batch(args):
    """c3: 64 independent simulations of uneven size advanced together, one graph launch of
    all their slice loops per 3D step, launch shapes picked by the autotuner; beside it the
    same simulations stepped one after another."""
    import numpy as np

    import qpad_gb300 as Q
    from qpad_gb300 import _capi as K
    prec = K.PREC_FP64 if args.precision == "fp64" else K.PREC_MIXED
    decks = Q.decks.c3()
    if args.slices:
        for d in decks:
            d.nz = args.slices
    sims = [Q.build_simulation(d, precision=prec) for d in decks]
    tune = [s.autotune(reps=10) for s in sims]
    pushes = sum(s.species[0].count() * d.nz for s, d in zip(sims, decks))
    batch = Q.Batch(sims)
    btune = batch.autotune(reps=1) if not args.no_autotune else None
    for _ in range(args.warmup):
        for s in sims:
            s.species[0].reset()
        batch.step()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        iters = []
        for _ in range(args.steps):
            for s in sims:
                s.species[0].reset()
            its = batch.step()
            iters.append(float(np.mean(np.concatenate(its))))
        wall = time.perf_counter() - t0
    value = pushes * args.steps / wall
    seq = None
    if not args.no_compare:                     # the same simulations one after another
        for s in sims:                          # with their single-simulation (latency) shapes
            s.autotune(reps=10)
            s.species[0].reset()
        t1 = time.perf_counter()
        for s in sims:
            s.run_3d_step()
        seq = pushes / (time.perf_counter() - t1)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == K.PREC_FP64 else "f32 particles / f64 solves",
        "data": "synthetic (seeded decks, no dataset)",
        "config": {"workload": f"c3_batch{len(decks)}_nz{decks[0].nz}", "simulations": len(decks),
                   "nr": sorted({d.nr for d in decks}), "max_mode": sorted({d.max_mode for d in decks}),
                   "plasma_pushes_per_step": pushes, "path": args.precision,
                   "l2": "step working set above L2 (64 simulations' stores and beams)"},
        "iters_per_slice": float(np.mean(iters)),
        "timing": "host wall clock around qpad_batch_step, which synchronises every simulation",
        "autotune": {"iter_cluster": sorted({t["iter_cluster"] for t in tune}),
                     "item_ppl": sorted({t["item_ppl"] for t in tune}), "batch": btune},
        "clocks": clk.summary(),
    }
    if seq is not None:
        line["sequential"] = {"value": seq, "speedup_of_batch": value / seq}
    print(json.dumps(line), flush=True)
    batch.close()
    for s in sims:
        s.close()
    return 0


def _traffic(deck, precision):
    """DRAM bytes per launch of the roofline kernels, copied from the committed ncu captures
    (profiles/dram_traffic_per_launch.json) for this workload, or {} when none was made."""
    tf = os.path.join(ROOT, "profiles", "dram_traffic_per_launch.json")
    try:
        wl = deck.name.split("_nz")[0].split("_beam")[0]
        return json.load(open(tf))["dram_bytes_per_launch"].get(wl, {}).get(precision, {})
    except Exception:
        return {}


def run_ours(args):
    import qpad_gb300 as Q
    from qpad_gb300 import _capi as K
    from qpad_gb300.diagnostics import step_error_report
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("gloo")
        torch.cuda.set_device(local)
    from qpad_gb300.replicas import replica_seed
    deck = _deck(args)
    deck.seed = replica_seed(deck.seed, rank)   # independent replica per GPU
    prec = K.PREC_FP64 if args.precision == "fp64" else K.PREC_MIXED
    inputs = Q.deck_inputs(deck)
    npl = len(inputs[0][4])
    nbeam = sum(len(b[2]) for b in inputs[1])
    want_err = not args.no_compare
    r = _measure(args, deck, inputs, prec, local, dist, args.steps, args.warmup, full=True, keep_stores=want_err,
                 order=args.guess_order)
    # the other arm of the metric: the plain FP64 path on the same deck and inputs
    cmp, err = None, None
    if not args.no_compare:
        other = K.PREC_FP64 if prec == K.PREC_MIXED else K.PREC_MIXED
        csteps = args.compare_steps or args.steps
        c = _measure(args, deck, inputs, other, local, dist, csteps, max(1, args.compare_warmup), full=False,
                     keep_stores=True)
        cmp = {"path": "fp64" if other == K.PREC_FP64 else "mixed", "value": c["value"],
               "ms_per_step": c["ms_per_step"], "iters_per_slice": c["iters_per_slice"],
               "graph": c["graph"]["active"], "steps": csteps, "warmup": max(1, args.compare_warmup)}
        ref_st, got_st = (c["stores"], r["stores"]) if other == K.PREC_FP64 else (r["stores"], c["stores"])
        err = step_error_report(got_st or {}, ref_st or {}, deck.max_mode)
        err["against"] = ("the plain FP64 GPU path on the same inputs, first 3D step (that path matches the FP64 "
                          "oracle within 1e-9 over whole steps in the parity tests)")
        ref_it, got_it = (c["first_iters"], r["first_iters"]) if other == K.PREC_FP64 else (r["first_iters"],
                                                                                          c["first_iters"])
        if got_it is not None and ref_it is not None:
            err["iters_per_slice_first_step"] = {"mixed": float(got_it.mean()), "fp64": float(ref_it.mean())}
        if prec == K.PREC_MIXED and not args.no_sensitivity and ref_st:
            # how much the deck amplifies round-off: the FP64 path run again from the same
            # inputs differs from the first run only by the order of its atomic additions
            # (FP64 round-off); the mixed path's error against FP32 unit round-off amplified
            # by the same factor says whether it is at the limit of FP32 particle state
            rep = step_error_report(_first_step_stores(args, deck, inputs, K.PREC_FP64, local), ref_st,
                                    deck.max_mode)
            amp = 2.0 ** -24 / 2.0 ** -53
            ratios = [v / (amp * rep["per_mode"][k]) for k, v in err["per_mode"].items()
                      if rep["per_mode"].get(k, 0.0) > 0.0]
            err["fp64_repeat"] = {"max": rep["max"], "worst": rep["worst"], "per_mode": rep["per_mode"],
                                  "what": "FP64 path run twice from the same inputs (atomic-order round-off), "
                                          "first step"}
            err["max_ratio_to_amplified_fp32_roundoff"] = max(ratios) if ratios else None
        r["stores"] = c["stores"] = None
    # the learned guess (trained nets for this deck's mode count), measured as its own arm
    learned = None
    if not args.no_compare and not args.no_learned:
        from qpad_gb300 import learned as LR
        wp = LR.weights_path(deck.max_mode)
        if os.path.exists(wp):
            lsteps = args.learned_steps or args.steps
            g = _measure(args, deck, inputs, prec, local, dist, lsteps, args.warmup, full=False, guess=True)
            learned = {"value": g["value"], "ms_per_step": g["ms_per_step"], "iters_per_slice": g["iters_per_slice"],
                       "iters_change": g["iters_per_slice"] / r["iters_per_slice"] - 1.0,
                       "weights": os.path.relpath(wp, ROOT), "steps": lsteps}
    kern = r["kern"]
    peak, peak_kind = _peaks()
    traffic = _traffic(deck, args.precision)
    # k_iterate: algorithmic bytes of one launch (every mode) -- it reads the raw deposits
    # (8 components), psi, B_old (2), b_beam (3), the factor rows of its three matrices and the
    # node tables; it writes the finished deposits (8), zeroes the raw ones (8), writes dJ/dxi
    # (2), b_spe, b, E (3 each), the convergence record and, on the mixed path, the FP32
    # gather table (6 floats per node and part)
    ld, P = deck.nr + 2, 2 * deck.max_mode + 1
    it_bytes = 8 * ((8 + 1 + 2 + 3) * P * ld + 9 * deck.nr * (deck.max_mode + 1) + 2 * ld) \
        + 8 * ((8 + 8 + 2 + 3 + 3 + 3) * P * ld + 2 * deck.nr) + (4 * 6 * P * ld if prec == K.PREC_MIXED else 0)
    it_ms, nit = kern["iterate"]
    it_avg_s = (it_ms / 1e3) / max(nit, 1)
    it_ach = it_bytes / it_avg_s / 1e9 if nit else None
    # the deposit: algorithmic bytes per particle of one amjdp pass: FP64 reads x, y, px, py,
    # pz, q and writes gamma, psi (64 B); mixed reads the cell word, two offsets, three
    # momenta, psi and q (28 B; psi only on the standard pusher, counted once here)
    amj_ms, namj = kern["amjdp"]
    bytes_per_particle = 64 if prec == K.PREC_FP64 else 28
    amj_avg_s = (amj_ms / 1e3) / max(namj, 1)
    achieved = bytes_per_particle * npl / amj_avg_s / 1e9 if namj else None
    it_roof = {"bound": "hbm", "achieved": it_ach, "peak": peak, "unit": "GB/s",
               "frac": (it_ach / peak) if it_ach else None, "traffic": traffic.get("k_iterate"),
               "kernel": "k_iterate", "peak_kind": peak_kind, "bytes_per_launch": it_bytes,
               "avg_launch_us": it_avg_s * 1e6, "device_ms_per_step": it_ms,
               "limiter": "latency: dependent FP64 chains and CTA/cluster barriers on an L2-resident "
                          "per-slice working set"}
    dep_name = "k_amjdp" if prec == K.PREC_FP64 else "k_mamjdp"
    dep_roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic.get(dep_name),
                "kernel": dep_name, "peak_kind": peak_kind, "bytes_per_launch": bytes_per_particle * npl,
                "avg_launch_us": amj_avg_s * 1e6, "device_ms_per_step": amj_ms,
                "limiter": "instruction issue (gather, push and 16 x (M+1) deposit sums per particle) and instruction fetch"}
    for rf in (it_roof, dep_roof):
        rf["traffic_source"] = ("copied from an ncu capture of a smaller cut of this workload with the same "
                                "per-slice work (profiles/dram_traffic_per_launch.json); not measured in this run"
                                if rf["traffic"] is not None else "no capture of this workload")
    # the dominant kernel of the step (by device time in the host-driven timing pass) is the
    # roofline line; the other beside it
    top_dep = amj_ms > it_ms
    dev_s = r["dev_s"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == K.PREC_FP64 else "f32 particles / f64 solves",
        "data": "synthetic (seeded deck, no dataset)",
        "config": {"workload": deck.name, "nr": deck.nr, "nz": deck.nz, "max_mode": deck.max_mode,
                   "plasma_particles_per_slice": npl, "beam_particles": nbeam, "path": args.precision,
                   "guess": (f"B-perp extrapolated from the previous slices, order {args.guess_order}"
                             if args.guess_order else "carried B-perp(j-1), as the reference"),
                   "iter_reltol": deck.iter_reltol, "iter_max": deck.iter_max,
                   "l2": "step working set above L2 (beam arrays and 3D field stores); per-slice data L2-resident",
                   "parallelism": f"replicas x{world}",
                   "cpu_sample": f"first {args.cpu_slices} slices (reference arm and cpu_baseline)"},
        "iters_per_slice": r["iters_per_slice"],
        "iteration_pushes_per_s": r["value"] * r["iters_per_slice"],
        "slices_per_s": world * deck.nz * args.steps / dev_s,
        "beam_pushes_per_s": world * nbeam * args.steps / dev_s,
        "wall_s": r["wall_s"],
        "e2e": r["e2e"],
        "gpu_launches": r["launches"],
        "roofline": dep_roof if top_dep else it_roof,
        "roofline_other": it_roof if top_dep else dep_roof,
        "clocks": r["clocks"],
        "graph": r["graph"],
        "autotune": r["tune"],
        "kernel_ms_per_step": {k: round(v[0], 3) for k, v in kern.items()},
        "kernel_launches_per_step": {k: v[1] for k, v in kern.items()},
    }
    if err is not None:
        line["max_mode_err"] = err["max"]
        line["max_mode_err_vs_field"] = err.get("max_vs_field")
        line["mode_err"] = err
    if learned is not None:
        line["learned_guess"] = learned
    if cmp is not None:
        line["compare"] = cmp
        line["speedup_vs_" + cmp["path"]] = r["value"] / cmp["value"]
        line["iters_change_vs_" + cmp["path"]] = r["iters_per_slice"] / cmp["iters_per_slice"] - 1.0
    if rank == 0 and not args.no_cpu_baseline:
        cs = CpuSample(deck)
        cb = max((cs.run(args.cpu_slices) for _ in range(2)), key=lambda x: x["value"])
        line["cpu_baseline"] = {"value": cb["value"], "unit": UNIT, "cores": cb["cores"], "kind": "port",
                                "iteration_pushes_per_s": cb["value"] * cb["iters_per_slice"],
                                "sample": cs.sample_text(cb["slices"]), "iters_per_slice": cb["iters_per_slice"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--deck", default="c5")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--guess-order", type=int, default=1, choices=[0, 1, 2],
                    help="initial B-perp guess of the measured arm: 0 carried (the reference), 1 / 2 extrapolated")
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-FP64 (or mixed) comparison arm")
    ap.add_argument("--compare-steps", type=int, default=1,
                    help="timed steps of the comparison arm (0: as --steps); its first warm-up step gives the error")
    ap.add_argument("--compare-warmup", type=int, default=1)
    ap.add_argument("--no-sensitivity", action="store_true",
                    help="skip the repeated FP64 run that measures how much the deck amplifies round-off")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-guess arm")
    ap.add_argument("--learned-steps", type=int, default=3, help="timed steps of the learned-guess arm (0: --steps)")
    ap.add_argument("--e2e-steps", type=int, default=5, help="steps of the end-to-end pass (at most --steps)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--item-ppl", type=int, default=0, choices=[0, 1, 2, 4],
                    help="particles per lane of the mixed deposit's work items (0: the autotuner's choice)")
    ap.add_argument("--cpu-slices", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--slices", type=int, default=0, help="override the deck's slice count (profiling runs)")
    ap.add_argument("--beam-frac", type=float, default=0.0, help="scale the beams' particle counts (profiling runs)")
    ap.add_argument("--graph", default="on", choices=["on", "off"],
                    help="off: host-driven slice loop (one launch per kernel, visible to per-kernel profilers)")
    args = ap.parse_args()
    if args.impl == "ours" and args.deck == "c3":
        return run_batch(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
