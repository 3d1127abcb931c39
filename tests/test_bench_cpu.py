"""bench.py's reference arm on the CPU: the FP64 oracle timed on the host cores
over a bounded sample of the default workload, printed as one JSON line with
the contract's keys; under torchrun only rank 0 works and prints."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = [sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-seconds", "1"]


def _run(extra_env=None):
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        env.pop(k, None)
    env.update(extra_env or {})
    return subprocess.run(ARGS, cwd=REPO, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_json_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # the line reports what was timed: the sample's cells and its own time per
    # step; the whole workload's figure is a separate, labelled projection
    n = d["config"]["cells"]
    assert n <= d["config"]["cells_in_workload"]
    assert abs(d["ms_per_step"] - 1e3 * n / d["value"]) <= 1e-6 * d["ms_per_step"]
    assert d["projected_ms_for_all_cells"] >= d["ms_per_step"]


def test_reference_arm_nonzero_rank_is_silent():
    r = _run({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
