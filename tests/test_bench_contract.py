"""bench.py's reference arm on the host (no GPU): the JSON line it prints carries the
keys of the benchmark contract, and under a multi-rank launch only rank 0 works and
prints.  The arm times the oracle (the CPU restatement of IrvingKirkwood::compute,
irvingkirkwood/IrvingKirkwood.h:74-110) on a bounded slice of a 2000-particle frame."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
        "--workload", "ik2d_n2k_g64_octic", "--steps", "2", "--warmup", "1"]


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    p = subprocess.run(ARGS, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    return p.stdout


def test_reference_arm_json_line():
    out = [ln for ln in _run({"WORLD_SIZE": "1", "RANK": "0"}).splitlines() if ln.strip()]
    assert len(out) == 1
    line = json.loads(out[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["unit"] == "frames/s" and line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"] == "ik2d_n2k_g64_octic"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1
    assert "whole frame" in cb["sample"]
    e2e = line["e2e"]
    assert e2e == {"value": line["value"], "unit": "frames/s",
                   "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the reference arm runs the oracle alone: none of the product's native libraries
    mapped = line["native_libraries_mapped"]
    assert mapped is not None and any(p.startswith("oracle") for p in mapped), mapped
    assert not any(p.startswith("pyglasstools_gb300") for p in mapped), mapped


def test_reference_arm_nonzero_rank_is_silent():
    assert _run({"WORLD_SIZE": "2", "RANK": "1"}).strip() == ""
