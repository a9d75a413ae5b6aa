"""The bench's workloads keep the configurations they are named for (CPU
only: nothing here launches a kernel).

  direct_n4096    plain direct sum, N = 4096, FP64, z in [0, 1] um
  bh_n65536       Barnes-Hut theta 0.5, leaf 16, N = 65,536, z in [0, 10] um
  fmm_n1m         FMM p = 8, N = 1,048,576, z in [0, 50] um
  batch256        256 plumes, FMM p = 6 above the direct threshold
  adjoint_n16384  N = 16,384, 50 leapfrog steps, checkpoint every 10

The per-plume generator (plume.make_plume) draws the distributions those
configurations describe; tests/test_oracle_golden.py pins it to the
reference's own plumes.
"""
import argparse
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

bench = pytest.importorskip("bench")


def test_workloads_match_their_configurations():
    w = bench.WORKLOADS
    d = w["direct_n4096"]
    assert (d["n"], d["precision"], d["length"]) == (4096, "fp64", 1e-6)
    b = w["bh_n65536"]
    assert (b["n"], b["theta"], b["leaf"], b["length"]) == (65536, 0.5, 16, 10e-6)
    f = w["fmm_n1m"]
    assert (f["n"], f["order"], f["length"]) == (1 << 20, 8, 50e-6)
    assert (w["batch256"]["nplumes"], w["batch256"]["order"]) == (256, 6)
    a = w["adjoint_n16384"]
    assert (a["n"], a["nsteps"], a["every"]) == (16384, 50, 10)


def test_default_run_is_the_headline_workload():
    """`python bench.py` with no flags runs the 1M-ion FMM workload on one GPU
    with at least 3 warm-up steps."""
    ap_parse = argparse.ArgumentParser.parse_args
    seen = {}

    def capture(self, args=None, namespace=None):
        seen["ns"] = ap_parse(self, [] if args is None else args, namespace)
        raise SystemExit(0)

    argparse.ArgumentParser.parse_args = capture
    argv = sys.argv
    try:
        sys.argv = ["bench.py"]
        with pytest.raises(SystemExit):
            bench.main()
    finally:
        sys.argv = argv
        argparse.ArgumentParser.parse_args = ap_parse
    ns = seen["ns"]
    assert ns.workload == "fmm_n1m" and ns.gpus == 1 and ns.warmup >= 3
