"""bench.py's output contract on the CPU: the reference arm (the oracle, timed on the host
cores) prints one JSON line with the keys of the benchmark line's contract, and the roofline
table covers the same kernels in both forms.  The reference arm runs here at ne4, the same
code path as its ne30 default."""
import json
import os
import subprocess
import sys

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--ne", "4",
                        "--steps", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    for k in ("metric", "value", "unit", "impl", "steps", "warmup", "higher_is_better", "config", "cpu_baseline",
              "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["unit"] == "SYPD" and line["value"] > 0
    assert line["warmup"] >= 3 and line["steps"] == 1 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["config"]["elements"] == 6 * 4 * 4


def test_roofline_table_covers_both_forms():
    t = bench.NCU_NE16
    assert set(t["fp64"]) == set(t["mixed"])
    for form in t:
        for k, (dram, flops, inst) in t[form].items():
            assert dram > 0 and flops >= 0 and inst >= 0 and flops >= inst, (form, k)
    # the per-launch figures scale with the element count
    row = bench.ncu_row("fp64", "caar_stage", 2 * bench.NCU_NE16_ELEMENTS, 10)
    assert row == tuple(2 * x for x in t["fp64"]["caar_stage"])


def test_sypd_of_an_interval():
    # one remap interval is 3 x 300 s of model time: 0.9 s of wall time per interval runs
    # the model 1000x faster than real time, 1000 / 365 simulated years per day
    assert abs(bench.sypd(1, 0.9) - 1000.0 / 365.0) < 1e-12
