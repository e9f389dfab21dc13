"""The reference arm of bench.py (the CPU oracle on the host cores) prints one JSON line with
the fields the benchmark contract names; a two-slice sample of the c1 deck keeps it short."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--cpu-slices", "2", "--deck", "c1"],
                         capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "vs_baseline",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True and d["config"]["workload"].startswith("c1")
    assert abs(d["iteration_pushes_per_s"] - d["value"] * d["iters_per_slice"]) <= 1e-9 * d["iteration_pushes_per_s"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_maps_only_the_oracle():
    """The reference arm's process draws its inputs from the oracle's loaders and never loads
    the product library."""
    code = ("import sys, bench\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--cpu-slices', '1',"
            " '--deck', 'c1']\n"
            "bench.main()\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libqpad_gpu' not in maps, 'product library mapped'\n"
            "assert 'libqpad_oracle' in maps\n")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]


def test_oracle_inputs_equal_product_inputs():
    """The reference arm's oracle-loaded deck equals the product loaders' deck bit for bit."""
    sys.path.insert(0, ROOT)
    import bench
    import qpad_gb300 as Q
    deck = Q.decks.c1().scaled(nz=32, beam_frac=0.01)
    _, pl, beams = bench.oracle_inputs(deck)
    (x, p, g, ps, q), qb = Q.deck_inputs(deck)
    for a, b in ((pl.x, x[:, 0]), (pl.y, x[:, 1]), (pl.px, p[:, 0]), (pl.pz, p[:, 2]), (pl.gamma, g), (pl.psi, ps),
                 (pl.q, q)):
        assert a.shape == b.shape and (a == b).all()
    for bm, (bx, bp, bq) in zip(beams, qb):
        assert bm.n == len(bq) and (bm.z == bx[:, 2]).all() and (bm.px == bp[:, 0]).all() and (bm.q == bq).all()
