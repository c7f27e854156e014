"""Flows in the layout of DiFfRG's generated code, compiled unchanged against the drop-in headers
and run on the GPU through the C++ integrators (tests/cpp/flow_driver.cu).

Each value (get and request, and for autodiff::real results value and derivative) is compared
with the FP64 oracle's restatement of the reference CPU integrator evaluating the same KERNEL
class on the host over the same quadrature, to 1e-12 relative to the integral of |integrand|.

* This repository's own generator-layout flows (tests/cpp/genflows: a seven-table vertex loop on
  IntegratorAngleGPU with RationalExpRegulator, a finite-T potential flow on IntegratorTBB<3> with
  double and autodiff::real results) always run.
* The reference's own generated flows -- Examples/YangMills/SP/flows/{AA/ZA, AAA/ZA3, AAAA/ZA4}.cu
  and Examples/ONfiniteT/flows/V/V.cu -- run when a DiFfRG checkout is available (read at test
  time from $GBINT_REFERENCE_DIR, never copied into this repository); otherwise they are skipped.
"""
import os
import re
import subprocess

import pytest

from conftest import reference_checkout

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GEN = os.path.join(HERE, "cpp", "genflows")
BIN = os.path.join(HERE, "cpp", "bin")

# (example dir relative to the checkout or None for this repository's flows, source, name, kind, oracle family)
OWN = [(None, "flows/loop/Zphi.cu", "Zphi", 1, 2), (None, "flows/V/Vt.cu", "Vt", 2, 1)]
REFERENCE = [("Examples/YangMills/SP", "flows/AA/ZA.cu", "ZA", 1, 2),
             ("Examples/YangMills/SP", "flows/AAA/ZA3.cu", "ZA3", 1, 4),
             ("Examples/YangMills/SP", "flows/AAAA/ZA4.cu", "ZA4", 1, 5),
             ("Examples/ONfiniteT", "flows/V/V.cu", "V", 2, 1)]


def _run(example_dir, source, name, kind, family, tag):
    from diffrg_gb300 import cppapi

    exe = cppapi.compile_flow(example_dir, source, name, kind, family, os.path.join(BIN, "flow_%s_%s" % (tag, name)))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=900)
    lines = r.stdout.strip().splitlines()
    assert lines and lines[-1].startswith("MAX"), r.stdout[-2000:] + r.stderr[-2000:]
    m = re.match(r"MAX (\S+) BAD (\d+)", lines[-1])
    assert r.returncode == 0 and m and int(m.group(2)) == 0, r.stdout[-3000:] + r.stderr[-2000:]
    values = [ln.split() for ln in lines[:-1]]
    assert len(values) >= 8
    for v in values:  # every result is a finite, non-trivial number
        gpu, host, scale = float(v[2]), float(v[3]), float(v[4])
        assert scale > 0 and abs(gpu) < 1e300
    return float(m.group(1))


@pytest.mark.parametrize("case", OWN, ids=[c[2] for c in OWN])
def test_generator_layout_flow_runs_and_matches_oracle(case):
    _, source, name, kind, family = case
    err = _run(GEN, source, name, kind, family, "gen")
    assert err <= 1e-12


@pytest.mark.parametrize("case", REFERENCE, ids=[c[2] for c in REFERENCE])
def test_reference_generated_flow_runs_and_matches_oracle(case):
    ref = reference_checkout()
    if ref is None:
        pytest.skip("no DiFfRG checkout (set GBINT_REFERENCE_DIR): the reference's flows are read, never copied")
    rel, source, name, kind, family = case
    err = _run(os.path.join(ref, rel), source, name, kind, family, "ref_" + rel.replace("/", "_"))
    assert err <= 1e-12
