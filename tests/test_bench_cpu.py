"""bench.py's JSON contract on the CPU: the reference arm (the oracle port of the reference's CPU
path on a bounded sample) prints one line with the keys the driver reads, on the same metric,
unit and workload as the GPU arm; the clock sampler summarises only the samples taken inside
the timed region (a stand-in nvidia-smi on PATH; no GPU)."""
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-n", "3000"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench
    assert d["metric"] == bench.METRIC and d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["scaling"] == "weak"
    assert d["config"]["particles"] == 1_000_000 and d["config"]["workload"].startswith("1,000,000-particle")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_clock_sampler_counts_only_the_timed_region(tmp_path):
    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\n"
                    "while true; do echo '0, 2070, 2070, 900.0, Active, Not Active, Not Active, Not Active, Active';"
                    " sleep 0.02; done\n")
    fake.chmod(0o755)
    env_path = os.environ.get("PATH", "")
    os.environ["PATH"] = f"{tmp_path}{os.pathsep}{env_path}"
    try:
        import bench
        with bench.ClockSampler(0) as c:
            time.sleep(0.2)
        got = c.summary()
    finally:
        os.environ["PATH"] = env_path
    assert got["sm_mhz"] == 2070.0 and got["sm_max_mhz"] == 2070.0
    assert got["reasons"] == ["sw_power_cap"]
    assert 3 <= got["samples"] <= 40
