"""Benchmark of the quasi-static slice loop (one JSON line on rank 0).

A step is one 3D step of the c2 deck: beam charge deposit, 1024 xi slices with the full
B-perp predictor-corrector (iter_reltol 1e-6), beam push, and the plasma renewal that
the reference performs after every 3D step.  The metric's first half, plasma
particle-pushes/s, is the headline value (one plasma particle advanced through one
slice, all of its predictor-corrector deposits included); B-perp iterations per slice
are reported beside it.  The headline path is the mixed-precision one (FP32 particles,
FP64 solves); the plain FP64 path runs on the same deck and inputs as the comparison arm
("compare", "speedup_vs_fp64", "iters_change_vs_fp64").

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--deck c2] [--precision mixed|fp64] [--no-compare]

--impl reference times the reference algorithm's CPU implementation (the project's C
restatement of it, OpenMP over particles, every host core) on a bounded sample of the
same deck; the Fortran reference itself cannot be built on these machines.
Multi-GPU runs are independent replicas (one simulation per GPU, different seeds).
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
    from qpad_gb300 import decks
    d = decks.DECKS[args.deck]()
    if args.slices:
        # profiling runs: the same slice workload over fewer slices
        d.nz = args.slices
        d.name = f"{d.name}_nz{args.slices}"
    return d


def cpu_sample(deck, nslices, steps=1, nthreads=None):
    """Times the oracle (C restatement of the reference loop, OpenMP over particles) on the
    first `nslices` slices of the deck with every plasma particle; the beam charge of the
    whole deck is deposited before the clock starts.  Returns pushes/s and details."""
    import numpy as np

    import qpad_gb300 as Q
    from oracle import oracle as O
    nthreads = nthreads or os.cpu_count()
    pl, beams = Q.deck_inputs(deck)
    g = O.grid(deck.nr, deck.nz, deck.max_mode, deck.dr, deck.dxi)
    x, p, gam, ps, q = pl
    opl = O.Plasma(len(q))
    opl.x[:], opl.y[:], opl.px[:], opl.py[:], opl.pz[:] = x[:, 0], x[:, 1], p[:, 0], p[:, 1], p[:, 2]
    opl.gamma[:], opl.psi[:], opl.q[:] = gam, ps, q
    sim = O.Sim(g, iter_max=deck.iter_max, iter_reltol=deck.iter_reltol, iter_abstol=deck.iter_abstol,
                dt3d=deck.dt, sp_npmax=len(q), beams=[(-1.0, O.PUSH3_REDUCED, len(b[2])) for b in beams],
                nthreads=nthreads)
    for k, (bx, bp, bq) in enumerate(beams):
        bm = O.Beam(len(bq))
        bm.x[:], bm.y[:], bm.z[:], bm.px[:], bm.py[:], bm.pz[:], bm.q[:] = (bx[:, 0], bx[:, 1], bx[:, 2],
                                                                               bp[:, 0], bp[:, 1], bp[:, 2], bq)
        sim.set_beam(k, bm)
    best, iters = None, []
    for _ in range(steps):
        sim.set_plasma(opl)
        sim.begin_3dstep()
        t0 = time.perf_counter()
        its = [sim.slice(j)[0] for j in range(1, nslices + 1)]
        t = time.perf_counter() - t0
        if best is None or t < best:
            best, iters = t, its
    pushes = len(q) * nslices
    return {"value": pushes / best, "seconds": best, "iters_per_slice": float(np.mean(iters)),
            "cores": nthreads, "slices": nslices, "particles_per_slice": len(q)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    deck = _deck(args)
    nslices = args.cpu_slices
    vals = []
    info = None
    for k in range(args.warmup + args.steps):
        info = cpu_sample(deck, nslices)
        if k >= args.warmup:
            vals.append(info["value"])
    v = statistics.median(vals)
    sample = (f"first {info['slices']} of {deck.nz} slices of {deck.name}, all {info['particles_per_slice']} "
              f"plasma particles, full predictor-corrector, beam charge precomputed")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": deck.name, "sample_slices": info["slices"]},
            "iters_per_slice": info["iters_per_slice"],
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": info["cores"], "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _measure(args, deck, inputs, prec, local, dist, full=True, guess=False):
    """Times args.steps 3D steps of one simulation (after args.warmup untimed ones) on the
    library's stream with CUDA events; with `full`, also the end-to-end pass with host
    buffers and one host-driven step with per-kernel event timing."""
    import qpad_gb300 as Q
    from qpad_gb300.replicas import reduce_timing
    sim = Q.build_simulation(deck, precision=prec, device=local, inputs=inputs)
    sim.use_graph(args.graph == "on")
    tune = sim.autotune(reps=20) if not args.no_autotune else None
    if guess:
        from qpad_gb300 import learned as LR
        from qpad_gb300.train_guess import DEFAULT_OUT
        nets = LR.load(DEFAULT_OUT, deck.max_mode, device=local)
        LR.attach(sim, *nets)
    sp = sim.species[0]
    npl = len(inputs[0][4])

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        sp.reset()
        sim.run_3d_step()
    barrier()
    sim.synchronize()
    sim.profile(True)
    l0 = sim.launch_count()
    iters_tot = 0
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
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
    dev_s, total_pushes = reduce_timing(dev_s, float(pushes_step * args.steps), dist)
    out = {"tune": tune, "value": total_pushes / dev_s, "ms_per_step": dev_s * 1e3 / args.steps,
           "iters_per_slice": iters_tot / (args.steps * deck.nz), "wall_s": wall, "launches": launches,
           "graph": {"active": graph_on, "status": graph_why}, "clocks": clk.summary(), "dev_s": dev_s,
           "pushes_step": pushes_step}
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
        # end to end through the C ABI with host buffers: renew from host arrays every step
        x, p, g, ps, q = inputs[0]
        h2d = sum(a.nbytes for a in (x, p, g, ps, q))
        d2h = 0
        e2e_t0 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            sp.renew(x, p, g, ps, q)
            it, _ = sim.run_3d_step()
            d2h += int(it.sum()) * 24 + 8
        e2e_s = time.perf_counter() - e2e_t0
        e2e_steps = max(1, args.steps)
        world = dist.get_world_size() if dist is not None else 1
        out["e2e"] = {"value": world * pushes_step * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h // e2e_steps}
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
                     "item_ppl": sorted({t["item_ppl"] for t in tune})},
        "clocks": clk.summary(),
    }
    if seq is not None:
        line["sequential"] = {"value": seq, "speedup_of_batch": value / seq}
    print(json.dumps(line), flush=True)
    batch.close()
    for s in sims:
        s.close()
    return 0


def run_ours(args):
    import qpad_gb300 as Q
    from qpad_gb300 import _capi as K
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
    r = _measure(args, deck, inputs, prec, local, dist, full=True)
    # the other arm of the metric: the plain FP64 path on the same deck and inputs
    cmp = None
    if not args.no_compare:
        other = K.PREC_FP64 if prec == K.PREC_MIXED else K.PREC_MIXED
        c = _measure(args, deck, inputs, other, local, dist, full=False)
        cmp = {"path": "fp64" if other == K.PREC_FP64 else "mixed", "value": c["value"],
               "ms_per_step": c["ms_per_step"], "iters_per_slice": c["iters_per_slice"],
               "graph": c["graph"]["active"]}
    # the learned guess (trained nets for the c2 shape), measured as its own arm
    learned = None
    if not args.no_compare and deck.name.startswith("c2") and deck.max_mode == 2:
        from qpad_gb300.train_guess import DEFAULT_OUT
        if os.path.exists(DEFAULT_OUT):
            g = _measure(args, deck, inputs, prec, local, dist, full=False, guess=True)
            learned = {"value": g["value"], "ms_per_step": g["ms_per_step"], "iters_per_slice": g["iters_per_slice"],
                       "iters_change": g["iters_per_slice"] / r["iters_per_slice"] - 1.0,
                       "weights": os.path.relpath(DEFAULT_OUT, ROOT)}
    kern = r["kern"]
    peak, peak_kind = _peaks()
    traffic = {}
    tf = os.path.join(ROOT, "profiles", "dram_traffic_per_launch.json")
    if os.path.exists(tf):
        try:
            # captured per workload; the profiling runs shorten the deck (same slice workload)
            wl = deck.name.split("_nz")[0]
            traffic = json.load(open(tf))["dram_bytes_per_launch"].get(wl, {}).get(args.precision, {})
        except Exception:
            traffic = {}
    # the dominant kernel, k_iterate: algorithmic bytes of one launch (every mode) -- it reads
    # the raw deposits (8 components), psi, B_old (2), b_beam (3), the factor rows of its three
    # matrices and the node tables; it writes the finished deposits (8), zeroes the raw ones
    # (8), writes dJ/dxi (2), b_spe, b, E (3 each), the convergence record and, on the mixed
    # path, the FP32 gather table (6 floats per node and part)
    ld, P = deck.nr + 2, 2 * deck.max_mode + 1
    it_bytes = 8 * ((8 + 1 + 2 + 3) * P * ld + 9 * deck.nr * (deck.max_mode + 1) + 2 * ld) \
        + 8 * ((8 + 8 + 2 + 3 + 3 + 3) * P * ld + 2 * deck.nr) + (4 * 6 * P * ld if prec == K.PREC_MIXED else 0)
    it_ms, nit = kern["iterate"]
    it_avg_s = (it_ms / 1e3) / max(nit, 1)
    it_ach = it_bytes / it_avg_s / 1e9 if nit else None
    # the deposit: algorithmic bytes per particle of one amjdp pass: FP64 reads x, y, px, py,
    # pz, q and writes gamma, psi (64 B); mixed reads the cell word, two offsets, three
    # momenta and q (28 B)
    amj_ms, namj = kern["amjdp"]
    bytes_per_particle = 64 if prec == K.PREC_FP64 else 28
    amj_avg_s = (amj_ms / 1e3) / max(namj, 1)
    achieved = bytes_per_particle * npl / amj_avg_s / 1e9 if namj else None
    dev_s = r["dev_s"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec == K.PREC_FP64 else "f32 particles / f64 solves",
        "data": "synthetic (seeded deck, no dataset)",
        "config": {"workload": deck.name, "nr": deck.nr, "nz": deck.nz, "max_mode": deck.max_mode,
                   "plasma_particles_per_slice": npl, "beam_particles": nbeam, "path": args.precision,
                   "iter_reltol": deck.iter_reltol, "iter_max": deck.iter_max,
                   "l2": "step working set above L2 (beam arrays and 3D field stores); per-slice data L2-resident",
                   "parallelism": f"replicas x{world}"},
        "iters_per_slice": r["iters_per_slice"],
        "slices_per_s": world * deck.nz * args.steps / dev_s,
        "beam_pushes_per_s": world * nbeam * args.steps / dev_s,
        "wall_s": r["wall_s"],
        "e2e": r["e2e"],
        "gpu_launches": r["launches"],
        "roofline": {"bound": "hbm", "achieved": it_ach, "peak": peak, "unit": "GB/s",
                     "frac": (it_ach / peak) if it_ach else None, "traffic": traffic.get("k_iterate"),
                     "kernel": "k_iterate", "peak_kind": peak_kind, "bytes_per_launch": it_bytes,
                     "avg_launch_us": it_avg_s * 1e6,
                     "limiter": "latency: dependent FP64 chains and CTA/cluster barriers on an L2-resident "
                                "per-slice working set"},
        "roofline_deposit": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": (achieved / peak) if achieved else None,
                             "traffic": traffic.get("k_amjdp" if prec == K.PREC_FP64 else "k_mamjdp"),
                             "kernel": "k_amjdp" if prec == K.PREC_FP64 else "k_mamjdp", "peak_kind": peak_kind,
                             "bytes_per_launch": bytes_per_particle * npl, "avg_launch_us": amj_avg_s * 1e6,
                             "limiter": "latency: particle and gather-table loads, one warp per cell work item"},
        "clocks": r["clocks"],
        "graph": r["graph"],
        "autotune": r["tune"],
        "kernel_ms_per_step": {k: round(v[0], 3) for k, v in kern.items()},
        "kernel_launches_per_step": {k: v[1] for k, v in kern.items()},
    }
    if learned is not None:
        line["learned_guess"] = learned
    if cmp is not None:
        line["compare"] = cmp
        line["speedup_vs_" + cmp["path"]] = r["value"] / cmp["value"]
        line["iters_change_vs_" + cmp["path"]] = r["iters_per_slice"] / cmp["iters_per_slice"] - 1.0
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_sample(deck, args.cpu_slices)
        line["cpu_baseline"] = {"value": cb["value"], "unit": UNIT, "cores": cb["cores"], "kind": "port",
                                "sample": f"first {cb['slices']} of {deck.nz} slices of {deck.name}, all "
                                          f"{cb['particles_per_slice']} plasma particles, OpenMP oracle"}
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
    ap.add_argument("--deck", default="c2")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-compare", action="store_true", help="skip the plain-FP64 (or mixed) comparison arm")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--cpu-slices", type=int, default=48)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--slices", type=int, default=0, help="override the deck's slice count (profiling runs)")
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
