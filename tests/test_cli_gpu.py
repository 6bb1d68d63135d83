"""The G2H command line end to end (main.cu:244-307): reference directory
layout in, the reference's CSV files out, for L4 and L3 labels."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("label", ["L4", "L3"])
def test_g2h_runs_and_writes_csvs(tmp_path, label):
    import gpuh2h
    from gpuh2h import _build
    _build.build()
    root = str(tmp_path)
    gpuh2h.generate_road(root, "cfg0")           # Graph/USA/cfg0*.txt, Partition/cfg0/Latitude*.txt
    env = dict(os.environ, H2H_QUERIES="20000", H2H_SEED="7", H2H_LABEL=label)
    args = [_build.CLI, "cfg0", "6", "2", "4", "1", "1", "2", "1"]
    # like the reference, the output directories must exist: without them the
    # run completes and reports the files it could not open
    r = subprocess.run(args, cwd=root, env=env, capture_output=True, timeout=300)
    assert r.returncode == 0 and b"Unable to open file for writing." in r.stderr
    os.makedirs(os.path.join(root, "ConstructInfo", "cfg0"))
    os.makedirs(os.path.join(root, "QueryResult", "cfg0"))
    r = subprocess.run(args, cwd=root, env=env, capture_output=True, timeout=300)
    assert r.returncode == 0, r.stderr.decode()
    out = r.stdout.decode()
    assert "connect!" in out and "n=4096" in out
    for f in ("ConstructInfo/cfg0/contract.csv", "ConstructInfo/cfg0/constructInfo.csv", "QueryResult/cfg0/random.csv"):
        p = os.path.join(root, f)
        assert os.path.exists(p), f
        lines = open(p).read().strip().split("\n")
        assert len(lines) >= 2, f                 # header + one row
        assert len(lines[1].split(",")) == len(lines[0].split(",")), f
    assert any(f.endswith("PartitionRate.csv") for f in os.listdir(root))
    # a CPU-only option is refused with a message, not a crash
    r2 = subprocess.run([_build.CLI, "cfg0", "6", "2", "4", "1", "0", "2", "1"], cwd=root, env=env,
                        capture_output=True, timeout=300)
    assert r2.returncode != 0 and b"contraction failed" in r2.stderr
