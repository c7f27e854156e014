"""The oracle reproduces the committed golden values of the benchmark workloads
(tests/golden/workloads_oracle.json, made by tests/golden/make_workload_golden.py)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def test_oracle_reproduces_workload_golden(oracle):
    import make_workload_golden as G

    want = json.load(open(G.OUT))
    got = G.generate()
    assert got["seeds"] == want["seeds"]
    for name, rec in want["workloads"].items():
        a = np.array([float(v) for v in rec["values"]])
        b = np.array([float(v) for v in got["workloads"][name]["values"]])
        assert a.shape == b.shape, name
        assert np.max(np.abs(a - b) / np.abs(a)) <= 1e-13, name
