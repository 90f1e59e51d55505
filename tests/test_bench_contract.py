"""The reference arm of bench.py (the float64 restatement timed on the host
cores) keeps the one-JSON-line contract, here on the small dense config.  No GPU."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None):
    env = dict(os.environ, **(extra_env or {}))
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "dense1k",
                           "--steps", "1", "--warmup", "3"],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)


def test_reference_arm_prints_one_contract_line():
    out = _run()
    assert out.returncode == 0, out.stderr
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == "logdet solves/s" and line["unit"] == "solves/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["steps"] == 1 and line["warmup"] >= 3
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "solves/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    out = _run({"RANK": "1"})
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""


def test_reference_arm_stops_timing_at_its_budget():
    # every timed step is a complete solve; past the budget no further step runs
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "dense1k",
                          "--steps", "3", "--warmup", "3", "--reference-budget-s", "0"],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["steps"] == 1 and line["steps_requested"] == 3
    assert abs(line["value"] - 1e3 / line["ms_per_step"]) <= 1e-9 * line["value"]


def test_roofline_of_fma_pipe_products():
    # fp32 / fp64 products are bounded by the FMA pipes, not the tensor cores
    sys.path.insert(0, ROOT)
    import bench

    prof = {c: {"ms": 0.0, "bytes": 0.0, "flops": 0.0, "launches": 0}
            for c in ("apply", "proj", "subproj", "sub", "scale", "quad", "other")}
    prof["apply"] = {"ms": 10.0, "bytes": 0.0, "flops": 7.2e9, "launches": 10}
    peaks = {"hbm": 6668.2, "tensor_burst": 1932.3, "tensor_sustained": 1729.1, "source": "measured"}
    rl = bench.roofline(prof, peaks, 1, "dense1k", "fp64")
    assert rl["bound"] == "fp64 fma" and rl["peak"] == 1.25
    assert abs(rl["achieved"] - 0.72) < 1e-9 and abs(rl["frac"] - 0.72 / 1.25) < 1e-12
    assert "nominal" in rl["peak_override"]
    rl32 = bench.roofline(prof, peaks, 1, "dense1k", "fp32")
    assert rl32["bound"] == "fp32 fma" and abs(rl32["peak"] - 152 * 256 * 2.07e9 / 1e12) < 1e-9
    rlt = bench.roofline(prof, peaks, 1, "rbf16k", "bf16x3")
    assert rlt["bound"] == "tensor" and rlt["peak"] == 1932.3
