"""Generate tests/golden/workloads_oracle.json: FP64 oracle values of fixed subsets of the
benchmark workloads C1-C5, with the seeds and generator rules they come from.

The inputs are the seeded synthetic workloads of diffrg_gb300/workloads.py and
diffrg_gb300/serving.py (numpy PCG64 streams, 5-point moving average along the momentum axis
with the window shrunk at the edges, FP32 table data).  The values are the oracle's
(oracle/, FP64 restatement of the reference CPU integrators) and pin both the oracle (CPU
test: it must reproduce them) and the GPU paths (GPU test: FP64 within 1e-12, FP32C within
1e-9).

    python tests/golden/make_workload_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "workloads_oracle.json")

# subsets: every integral of C1, a spread of the others
SUBSETS = {
    "C1": list(range(64)),
    "C2": [0, 17, 63, 127, 128, 150, 200, 255, 256, 300, 350, 383],
    "C3": [0, 1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233, 377, 610, 987, 1597, 2584, 4095],
    "C5": [0, 21, 63, 64, 100, 127],
}
C4_PAIRS = [(0, 0), (0, 64), (1, 5), (1, 127), (2, 30), (7, 90), (16, 3), (31, 127)]
C4_K = 0.7


def generate():
    from diffrg_gb300 import serving, workloads
    from oracle import oracle as O

    O.build()
    out = {"rng": "numpy.random.default_rng(seed) (PCG64)", "seeds": workloads.SEEDS,
           "smoothing": "5-point moving average along the first axis, window shrunk to the existing points at the ends",
           "workloads": {}}
    for name, sub in SUBSETS.items():
        w = getattr(workloads, name.lower())()
        vals = workloads.oracle_values(w, O, subset=sub)
        out["workloads"][name] = {"subset": sub, "values": [repr(float(v)) for v in vals]}
    w4 = serving.c4()
    vals = serving.oracle_subset(O, w4, w4["y0"], C4_K, C4_PAIRS)
    out["workloads"]["C4"] = {"k": C4_K, "pairs": C4_PAIRS, "values": [repr(float(v)) for v in vals]}
    return out


def main():
    out = generate()
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
