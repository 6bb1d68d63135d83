"""The G2H command line end to end (main.cu:244-307): reference directory
layout in, the reference's CSV files out, for L4 and L3 labels."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

# The reference's CSV header lines, byte for byte: contract.csv and
# constructInfo.csv share one header (TreeStructure.cu:77,
# Graph_Fundamental.cu:148, with its two empty columns), random.csv has the
# query-timing header (Query.cu:608).
CONSTRUCT_HEADER = (
    "graphName,PartitionTreeHeight,changeHeight,ParititionTime,makePartitionRankTreeTime,AlllocateLUBTime,LUBSize,"
    "translateLUBToGPUTime,TDInGPUTime,translateBackAndMallocToCPUTime,vertexesConstructedInGPU,"
    "DecompositionTreeSize,TDInCPUTime,TDTREEHeight,,RMQsize,translateRMQTime,H2HLabelSize,,"
    "changeConstructDeviceSize,H2HmallocTime,H2HConstructBFSTreeTime,H2HTranslateBFSTreeTime,H2HUsingTime_CPU,"
    "H2HTranslateTime,H2HUsingTime_GPU,PartitionMethod,threadNum,contractDevice,parallelFine,constructDevice")
QUERY_HEADER = (
    "queryNumber,sequence,multiThread-4,multiThread-6,multiThread-8,multiThread-10,multiThread-12,multiThread-14,"
    "multiThread-16,GPUnoLCA-64,GPUwithLCA-64,GPUnoLCA-128,GPUwithLCA-128,GPUnoLCA-256,GPUwithLCA-256,"
    "GPUnoLCA-512,GPUwithLCA-512,GPUnoLCA-1024,GPUwithLCA-1024,TreeHeight,changeHeight,PartitionMethod,"
    "contractDevice")


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
    for f, header in (("ConstructInfo/cfg0/contract.csv", CONSTRUCT_HEADER),
                      ("ConstructInfo/cfg0/constructInfo.csv", CONSTRUCT_HEADER),
                      ("QueryResult/cfg0/random.csv", QUERY_HEADER)):
        p = os.path.join(root, f)
        assert os.path.exists(p), f
        raw = open(p, "rb").read()
        assert raw.startswith((header + "\n").encode()), f   # the header line, byte for byte
        lines = raw.decode().strip().split("\n")
        assert len(lines) >= 2, f                 # header + one row
        assert len(lines[1].split(",")) == len(lines[0].split(",")), f
    assert any(f.endswith("PartitionRate.csv") for f in os.listdir(root))
    # a CPU-only option is refused with a message, not a crash
    r2 = subprocess.run([_build.CLI, "cfg0", "6", "2", "4", "1", "0", "2", "1"], cwd=root, env=env,
                        capture_output=True, timeout=300)
    assert r2.returncode != 0 and b"contraction failed" in r2.stderr
