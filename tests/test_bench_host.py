"""Host side of bench.py (no GPU): the reference arm's BCP and full-scan lines
on a small workload, the algorithmic-byte formula, and the recorded DRAM
traffic being used only for the exact workload and launch shape it was
measured on."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def run_bench(*args):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_bcp_line(orc):
    d = run_bench("--impl", "reference", "--n-vars", "3000", "--trails", "96", "--steps", "2", "--warmup", "1",
                  "--cpu-trails", "64", "--ref-own-trails", "32", "--no-solve", "--no-latency")
    assert d["impl"] == "reference" and d["metric"] == "BCP props/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["e2e"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    own = d["cpu_baseline"]["ref_own_scaled"]
    assert "unavailable" in own or (own["kind"] == "reference" and own["value"] > 0)


def test_reference_arm_full_scan_line(orc):
    d = run_bench("--workload", "full_scan", "--impl", "reference", "--n-vars", "2000", "--trails", "64",
                  "--steps", "2", "--warmup", "1", "--cpu-trails", "32")
    assert d["impl"] == "reference" and d["unit"] == "evaluations/s" and d["value"] > 0


def test_algorithmic_bytes_and_recorded_traffic():
    sys.path.insert(0, str(ROOT))
    import bench
    cnt = np.zeros((2, 6), np.int64)
    cnt[:, 1:] = [[10, 30, 25, 2, 7], [0, 0, 0, 0, 3]]   # W, L, A, I, T per trail
    assert bench.alg_bytes(cnt) == 4 * 10 + 4 * 30 + 25 + 9 * 2 + 5 * 10
    rec = json.loads((ROOT / "profiles" / "bcp_traffic.json").read_text())
    key = (rec["n_vars"], rec["n_trails"], rec["window"], rec["slots"], rec.get("order_pivot", 0))
    assert bench.traffic_per_launch(*key) == rec["dram_bytes_per_launch"]
    # any other workload or launch shape has no recorded traffic
    assert bench.traffic_per_launch(key[0], key[1], key[2], key[3], key[4] + 1) is None
    assert bench.traffic_per_launch(key[0] // 2, *key[1:]) is None
