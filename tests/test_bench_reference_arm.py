"""The reference arm of bench.py (`--impl reference`) runs on the host alone
and prints one JSON line of the contract, in the same metric and units as our
arm: the reference itself built from its sources (oracle/_ref/ref_harness)
on every host core where it is built and runs the workload, else the oracle
port of its CPU path."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


@pytest.mark.parametrize("workload", ["rpm16k", "dipoles"])
def test_reference_arm_line(workload):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", workload, "--steps", "1",
                        "--warmup", "1", "--ref-seconds", "0.3"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "trial moves/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 1
    built = os.path.exists(os.path.join(ROOT, "oracle", "_ref", "ref_harness"))
    want = "reference" if built and workload != "dipoles" else "port"
    assert d["cpu_baseline"]["kind"] == want and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["metric"].startswith("MC trial moves/s")
