"""The bench's reference arm (the reference's CPU path, here its C
restatement, on the host cores) keeps the JSON contract: one line with the
same metric and workload as the GPU arm, `impl` = "reference", a
`cpu_baseline` describing the run and an `e2e` with no host-device copies.
Run on a 32^3 lattice so that it takes a second."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--lattice", "32"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("time to max|F|<1e-6 & site-steps/s")
    assert d["unit"] == "site-steps/s" and d["higher_is_better"] is True and d["dtype"] == "f64"
    assert d["value"] > 0 and d["steps"] == 2
    assert d["config"]["workload"].startswith("32^3 lattice, homeotropic z-walls (planes 0 and 31)")
    assert d["config"]["sites"] == 32 ** 3
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and "32^3" in cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
