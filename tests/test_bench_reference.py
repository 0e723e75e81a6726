"""The reference arm of bench.py, on the CPU: lair's getrf_row_major + getrs
(the oracle's C++ restatement, one thread) timed on a bounded slice of the
workload, printed as one JSON line with the bench contract's keys; under a
multi-rank launch only rank 0 prints."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_reference(env_extra, *args):
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    env.update(env_extra)
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def json_lines(stdout):
    return [json.loads(line) for line in stdout.splitlines() if line.startswith("{")]


def test_reference_arm_prints_the_contract_line():
    r = run_reference({}, "--steps", "2", "--warmup", "1", "--n", "1024", "--ref-elim-steps", "3")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "GFLOP/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1 and d["dtype"] == "f64"
    assert d["config"]["n"] == 1024
    cpu = d["cpu_baseline"]
    assert cpu["value"] == d["value"] and cpu["kind"] == "port" and cpu["cores"] == 1 and cpu["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = run_reference({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--steps", "1", "--warmup", "0",
                      "--n", "256")
    assert r.returncode == 0, r.stderr[-2000:]
    assert json_lines(r.stdout) == []


def test_roofline_traffic_comes_from_the_committed_profiles():
    """The bench's roofline.traffic is the per-launch DRAM traffic of the
    dominant kernel from its committed ncu summary (both update engines)."""
    sys.path.insert(0, ROOT)
    import bench

    for name in ("oz_gemm_fp64_slices_n16384.md", "gemm_dmma_persistent_fp64_n16384.md"):
        t = bench.read_traffic(os.path.join(ROOT, "profiles", name))
        assert t is not None and t > 1e9, name
    assert bench.read_traffic(os.path.join(ROOT, "profiles", "no_such_profile.md")) is None
