"""Build helper for programs that use the C++ class templates (include/gbint/integrators.hh).

A user translation unit that includes the header is compiled by nvcc for sm_103a and linked
against the in-tree libgbint.so; `compile_program` does exactly that (with an rpath to the
library), `build_tests` compiles the test driver tests/cpp/test_integrators.cu, and
`compile_flow` compiles a flow in the layout of DiFfRG's generated code (an example directory
holding flows/def.hh and flows/<dir>/<X>.{hh,cu,kernel}) into tests/cpp/flow_driver.cu with the
drop-in headers at the reference's include paths (include/gbint/compat).
"""
from __future__ import annotations

import hashlib
import os
import subprocess

from . import build as B

ROOT = B.ROOT
TEST_SRC = os.path.join(ROOT, "tests", "cpp", "test_integrators.cu")
TEST_BIN = os.path.join(ROOT, "tests", "cpp", "bin", "test_integrators")


COMPAT = os.path.join(B.INCLUDE, "gbint", "compat")
FLOW_DRIVER = os.path.join(ROOT, "tests", "cpp", "flow_driver.cu")
ORACLE_DIR = os.path.join(ROOT, "oracle")


def _headers_digest(h) -> None:
    for d, _, fs in sorted(os.walk(B.INCLUDE)):
        for f in sorted(fs):
            if f.endswith((".h", ".hh", ".cuh")):
                h.update(f.encode())
                h.update(open(os.path.join(d, f), "rb").read())


def compile_flow(example_dir: str, source: str, name: str, kind: int, family: int, out: str) -> str:
    """Compile tests/cpp/flow_driver.cu around the flow file `source` (relative to example_dir,
    e.g. "flows/AA/ZA.cu"); the flow's own files are compiled as they are."""
    lib = B.build()
    libdir = os.path.dirname(lib)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    h = hashlib.sha256()
    _headers_digest(h)
    for p in (FLOW_DRIVER, os.path.join(ORACLE_DIR, "families.hh"), os.path.join(ORACLE_DIR, "oracle.hh")):
        h.update(open(p, "rb").read())
    flows = os.path.join(example_dir, "flows")
    for d, _, fs in sorted(os.walk(flows)):
        for f in sorted(fs):
            h.update(open(os.path.join(d, f), "rb").read())
    h.update(("%s|%s|%d|%d" % (source, name, kind, family)).encode())
    h.update(open(lib, "rb").read()[:4096])
    stamp = out + ".stamp"
    if os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return out
    cmd = [B.nvcc(), "-std=c++20", "-O2", "--expt-relaxed-constexpr", "-I", COMPAT, "-I", B.INCLUDE, "-I", ORACLE_DIR,
           "-I", example_dir, '-DGBINT_FLOW_SOURCE="%s"' % source, "-DGBINT_FLOW_NAME=%s" % name,
           "-DGBINT_FLOW_KIND=%d" % kind, "-DGBINT_FLOW_FAMILY=%d" % family] + B.ARCH + \
        [FLOW_DRIVER, "-o", out, "-L", libdir, "-lgbint", "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stderr[-6000:])
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    return out


def compile_program(src: str, out: str, extra=()) -> str:
    lib = B.build()
    libdir = os.path.dirname(lib)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    h = hashlib.sha256()
    h.update(open(src, "rb").read())
    _headers_digest(h)
    extra = list(extra)
    for i, a in enumerate(extra):  # the files of extra include directories (e.g. a flows/ tree)
        if a == "-I" and i + 1 < len(extra) and os.path.isdir(extra[i + 1]) and not extra[i + 1].startswith(B.INCLUDE):
            for d, _, fs in sorted(os.walk(extra[i + 1])):
                for f in sorted(fs):
                    h.update(open(os.path.join(d, f), "rb").read())
    h.update(" ".join(extra).encode())
    h.update(open(lib, "rb").read()[:4096])
    stamp = out + ".stamp"
    if os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == h.hexdigest():
        return out
    cmd = [B.nvcc(), "-std=c++17", "-O2", "-lineinfo", "--expt-relaxed-constexpr", "-I", B.INCLUDE] + B.ARCH + \
          list(extra) + \
          [src, "-o", out, "-L", libdir, "-lgbint", "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stderr[-6000:])
    with open(stamp, "w") as f:
        f.write(h.hexdigest())
    return out


def build_tests() -> str:
    return compile_program(TEST_SRC, TEST_BIN)


QMC_SRC = os.path.join(ROOT, "tests", "cpp", "test_qmc.cu")
QMC_BIN = os.path.join(ROOT, "tests", "cpp", "bin", "test_qmc")


def build_qmc_tests() -> str:
    """The QMC integrators' test driver, compiled through the reference's header paths."""
    return compile_program(QMC_SRC, QMC_BIN, extra=["-std=c++20", "-I", COMPAT])


DROPIN_SRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bench", "dropin_bench.cu")
DROPIN_BIN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bench", "bin", "dropin_bench")


def build_dropin_bench() -> str:
    """The C++ drop-in benchmark (bench.py's cpp_dropin leg): the generator-layout vertex loop of
    tests/cpp/genflows through the drop-in headers, compiled as a user translation unit."""
    return compile_program(DROPIN_SRC, DROPIN_BIN,
                           extra=["-std=c++20", "-I", COMPAT, "-I", os.path.join(ROOT, "tests", "cpp", "genflows")])
