"""Build helper for programs that use the C++ class templates (include/gbint/integrators.hh).

A user translation unit that includes the header is compiled by nvcc for sm_103a and linked
against the in-tree libgbint.so; `compile_program` does exactly that (with an rpath to the
library), `build_tests` compiles the test driver tests/cpp/test_integrators.cu.
"""
from __future__ import annotations

import hashlib
import os
import subprocess

from . import build as B

ROOT = B.ROOT
TEST_SRC = os.path.join(ROOT, "tests", "cpp", "test_integrators.cu")
TEST_BIN = os.path.join(ROOT, "tests", "cpp", "bin", "test_integrators")


def compile_program(src: str, out: str, extra=()) -> str:
    lib = B.build()
    libdir = os.path.dirname(lib)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    h = hashlib.sha256()
    for p in (src, os.path.join(B.INCLUDE, "gbint.h"), os.path.join(B.INCLUDE, "gbint", "integrators.hh"),
              os.path.join(B.INCLUDE, "gbint", "interpolators.hh"), os.path.join(B.INCLUDE, "gbint", "autodiff.hh"),
              os.path.join(B.INCLUDE, "gbint", "regulators.hh"),
              os.path.join(B.INCLUDE, "gbint", "flow_utils.hh"),
              os.path.join(B.INCLUDE, "gbint", "kernel_math.hh"),
              os.path.join(B.INCLUDE, "gbint", "device", "families.cuh")):
        h.update(open(p, "rb").read())
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
