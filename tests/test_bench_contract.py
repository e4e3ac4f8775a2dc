"""The benchmark's reference arm runs on host cores only, so its JSON line is
checked here on the CPU: the keys and meanings every bench line carries, the
reference arm's own `impl`, `cpu_baseline` and zero-copy `e2e`, and that a
non-zero rank under a multi-process launch exits 0 without work."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def run_bench(extra_env: dict, *args: str) -> subprocess.CompletedProcess:
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    env.update(extra_env)
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_line():
    p = run_bench({}, "--impl", "reference", "--config", "1", "--steps", "1", "--warmup", "1")
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in line, key
    assert line["unit"] == "bases/s" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert "workload" in line["config"] and line["vs_baseline"] is None
    # the same config dict as the GPU arm's line for the same workload
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    bench.WORKLOAD, bench.K, bench.CUTOFF, bench.DESC = bench.CONFIGS[1]
    assert line["config"] == bench.config_dict()
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["kind"] in ("port", "reference")
    assert cpu["cores"] >= 1 and cpu["sample"]
    assert "whole workload" in cpu["sample"]  # no prefix sample under the full workload's config
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    p = run_bench({"RANK": "1", "WORLD_SIZE": "2"}, "--impl", "reference", "--steps", "1", "--warmup", "1")
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
