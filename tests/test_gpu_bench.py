"""The GPU arm of the benchmark: one JSON line with the contract's keys
(device value, end-to-end value with its host<->device bytes, roofline,
clocks, kernel launches)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.gpu
def test_bench_line_keeps_the_contract():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--steps", "1", "--warmup", "3",
                          "--no-cpu-baseline", "--no-time-to-gap", "--no-other-workloads"], capture_output=True, text=True, timeout=900,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["unit"] == "ant-tours+LS/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3 and d["scaling"] == "weak"
    assert d["ms_per_step"] > 0 and d["vs_baseline"] is None and d["data"] == "synthetic"
    assert d["config"]["iterations_per_step"] == 16 and d["config"]["timed_iterations"] == [0, 16]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    roof = d["roofline"]
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and roof["peak"] > 0
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-9 and roof["traffic"] > 0
    # the roofline describes the timed window: its bytes over the timed step time
    assert abs(roof["achieved"] * 1e9 * d["ms_per_step"] / 1e3 - roof["bytes_per_step"]) < 1e-6 * roof["bytes_per_step"]
    assert 0 < roof["ant_kernel"]["share_of_unchained_time"] < 1
    assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
    plan_launches = d["gpu_launches"]
    assert plan_launches == 16 * 16 * 1        # 8 chains x (ant launch + update) x 16 iterations x 1 step
    assert d["steady_state"]["value"] > 0
