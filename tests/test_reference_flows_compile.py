"""CPU: the reference's generated flows compile UNCHANGED against the drop-in headers.

DiFfRG's code generator writes each example's flows/ directory: def.hh (includes
DiFfRG/common/utils.hh and DiFfRG/physics/{integration,integration_finiteT,interpolation,
regulators,thermodynamics}.hh), one <X>.hh/.cu/.kernel triple per flow, and flows.cc (the
FlowEquations subclass).  Read at test time from a DiFfRG checkout ($GBINT_REFERENCE_DIR, or a
'reference' directory beside this repository; skipped when absent), never copied:

* every flow .cu that an example's flows/CMakeLists.txt builds is compiled by nvcc for sm_103a
  with include/gbint/compat first on the include path (the examples' KERNEL device code, the
  integrator templates and their fused kernels included) -- the ten FourFermi flows take one to
  four minutes each, so they join only with GBINT_REFERENCE_FLOWS_ALL=1;
* every example's flows.cc is compiled by the host compiler (g++), as the reference's build
  compiles it, and by nvcc.
This repository's own generator-layout flows (tests/cpp/genflows) compile in every run.  nvcc
cross-compiles without a GPU; nothing runs.
"""
import concurrent.futures as cf
import os
import re
import shutil
import subprocess

import pytest

from diffrg_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))
COMPAT = os.path.join(B.INCLUDE, "gbint", "compat")
EXAMPLES = ["YangMills/SP", "YangMills/Full", "ONfiniteT", "QuarkMesonLPAprime", "FourFermi"]
SLOW = ("FourFermi",)


def _nvcc(src, obj, inc, lang=()):
    cmd = [B.nvcc(), "-std=c++20", "-O1", "--expt-relaxed-constexpr", "-I", COMPAT, "-I", B.INCLUDE, "-I", inc] + \
        list(lang) + B.ARCH + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stderr[-3000:]


def _gxx(src, obj, inc):
    cuda = os.path.dirname(os.path.dirname(B.nvcc()))
    cmd = [shutil.which("g++") or "g++", "-std=c++20", "-O1", "-I", COMPAT, "-I", B.INCLUDE, "-I", inc,
           "-I", os.path.join(cuda, "include"), "-I", os.path.join(cuda, "include", "cccl"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stderr[-3000:]


def _built_flows(example):
    """The .cu flows an example's flows/CMakeLists.txt lists for its CUDA build."""
    txt = open(os.path.join(example, "flows", "CMakeLists.txt")).read()
    cuda_part = txt.split("else()")[0]
    return [os.path.join(example, p) for p in re.findall(r"(flows/[A-Za-z0-9_/]+\.cu)", cuda_part)]


def _run_all(jobs):
    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        res = list(ex.map(lambda j: j[0](*j[1:]), jobs))
    bad = [(s, e) for s, rc, e in res if rc != 0]
    assert not bad, "\n\n".join("%s\n%s" % b for b in bad)
    return len(res)


def test_reference_generated_flows_compile_unchanged(reference_dir, tmp_path):
    allflows = os.environ.get("GBINT_REFERENCE_FLOWS_ALL") == "1"
    jobs = []
    for ex in EXAMPLES:
        exdir = os.path.join(reference_dir, "Examples", ex)
        if not os.path.isdir(exdir):
            continue
        flows_cc = os.path.join(exdir, "flows", "flows.cc")
        tag = ex.replace("/", "_")
        jobs.append((_gxx, flows_cc, str(tmp_path / (tag + "_flows_gxx.o")), exdir))
        jobs.append((_nvcc, flows_cc, str(tmp_path / (tag + "_flows_nvcc.o")), exdir, ("-x", "cu")))
        if ex in SLOW and not allflows:
            continue
        for src in _built_flows(exdir):
            obj = str(tmp_path / (tag + "_" + os.path.basename(src) + ".o"))
            jobs.append((_nvcc, src, obj, exdir))
    # the long ones first, so that they overlap the many short ones
    jobs.sort(key=lambda j: 0 if "AAAA" in j[1] or "FourFermi" in j[1] else 1)
    n = _run_all(jobs)
    assert n >= 18 + 10


def test_own_generator_layout_flows_compile(tmp_path):
    gen = os.path.join(HERE, "cpp", "genflows")
    jobs = [(_nvcc, os.path.join(gen, "flows", "loop", "Zphi.cu"), str(tmp_path / "Zphi.o"), gen),
            (_nvcc, os.path.join(gen, "flows", "V", "Vt.cu"), str(tmp_path / "Vt.o"), gen)]
    assert _run_all(jobs) == 2
