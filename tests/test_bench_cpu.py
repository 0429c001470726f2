"""bench.py's reference arm and JSON contract, on the CPU.

`bench.py --impl reference` times the reference's CPU algorithm (the oracle
restatement) on the host cores and prints one JSON line with the same
metric, unit and workload as the GPU arm, plus `impl`, `cpu_baseline` and an
`e2e` entry with no transfers.  Checked here for the default run (every
workload, C5 the headline with the others under `configs`) and for C1 alone,
with short CPU samples.
"""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _reference_line(*extra):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
           "--warmup", "1", "--cpu-seconds", "0.3", "--cpu-seconds-other", "0.2", *extra]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


@pytest.mark.parametrize("workload", [None, "c1"])
def test_reference_arm_contract(workload):
    d = _reference_line(*([] if workload is None else ["--workload", workload]))
    assert d["impl"] == "reference"
    if workload is None:
        assert d["config"]["workload"].startswith("c5")
        assert sorted(d["configs"]) == ["c1", "c2", "c3", "c4", "c5"]
        for name, c in d["configs"].items():
            assert c["impl"] == "reference" and c["value"] > 0, name
            assert c["config"]["workload"] == name
    else:
        assert d["config"]["workload"] == workload
    assert d["unit"] == "Gpoint*modes/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_clock_summary(tmp_path, monkeypatch):
    """The clock record: median SM clock, max clock, throttle reasons seen."""
    sys.path.insert(0, ROOT)
    import bench
    csv = tmp_path / "clocks.csv"
    csv.write_text("0, 1965, 2070, 810.5, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                   "0, 2040, 2070, 1210.0, 0x4, Not Active, Not Active, Not Active, Active\n"
                   "0, 2010, 2070, [N/A], 0x0, Not Active, Not Active, Not Active, Not Active\n"
                   "garbage\n")
    monkeypatch.delenv("GSC_CLOCKS_CSV", raising=False)
    s = bench.ClockSampler(0)
    s.path, s.proc = str(csv), object()
    d = s.summary()
    assert d["sm_mhz"] == 2010.0 and d["sm_max_mhz"] == 2070.0 and d["samples"] == 3
    assert d["reasons"] == ["sw_power_cap"] and d["power_w_max"] == 1210.0
    assert not csv.exists()                      # temporary samples are removed
