"""bench.py --impl reference (the CPU oracle of the same step, no GPU) keeps the bench
line's contract: one JSON line from rank 0 with the engine arm's metric, unit and
direction, the number of steps it actually timed, `impl`, a `cpu_baseline` describing the
run and an `e2e` with no host-device bytes; other ranks print nothing.  Run on the 64 x 64
unit-square workload (8,192 triangles), where an oracle step takes milliseconds."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(*args, env=None):
    e = dict(os.environ, OMP_NUM_THREADS="2")
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "square",
                        *args], capture_output=True, text=True, env=e, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]


def test_reference_arm_line():
    lines = _bench("--steps", "3", "--warmup", "1", "--ref-budget", "60")
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["metric"] == "ms per PFEM-2 step" and d["unit"] == "ms/step"
    assert d["higher_is_better"] is False and d["n_gpus"] == 1 and d["dtype"] == "f64"
    assert d["steps"] == 3 and d["warmup"] == 1 and d["value"] > 0 and d["ms_per_step"] == d["value"]
    assert d["config"]["same_config_as_engine_arm"] is True and d["config"]["timed_from_step"] == 2
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] == 2 and "3 oracle step(s)" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["reference_algorithms"]["ms_per_step"] > 0


def test_reference_arm_reports_the_steps_it_timed():
    # a budget that one step already exhausts: exactly one step is timed and reported
    d = _bench("--steps", "20", "--warmup", "0", "--ref-budget", "0", "--ref-algorithms", "0")[0]
    assert d["steps"] == 1 and d["config"]["steps_requested"] == 20 and "reference_algorithms" not in d


def test_reference_arm_prints_on_rank_zero_only():
    assert _bench("--steps", "1", "--warmup", "0", env={"RANK": "1", "WORLD_SIZE": "2"}) == []
