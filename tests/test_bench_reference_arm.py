"""bench.py --impl reference on the CPU: the arm runs the oracle's
restatement of the reference's CPU path on the 264,346-vertex graph, prints
one JSON line with the contract's keys, and its process maps no library of
this repository but the oracle's (it must not time or load the product)."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SNIPPET = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    if e.code not in (0, None):
        raise
with open("/proc/self/maps") as f:
    libs = sorted({line.split()[-1] for line in f if line.rstrip().endswith(".so")})
print("MAPS " + " ".join(libs))
"""


def test_reference_arm_line_and_libraries():
    from oracle import oracle
    oracle.build()  # the arm needs the oracle library (built here when absent)
    r = subprocess.run([sys.executable, "-c", SNIPPET], cwd=REPO, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "queries/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "why_not_road6m" in d["config"]
    maps = [ln for ln in r.stdout.splitlines() if ln.startswith("MAPS ")][0].split()[1:]
    ours = [p for p in maps if p.startswith(REPO)]
    assert ours, "the oracle library was not loaded"
    assert all(os.sep + "oracle" + os.sep in p for p in ours), ours
    assert not any("libgpuh2h" in p for p in maps), maps
