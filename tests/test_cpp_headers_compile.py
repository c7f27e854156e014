"""CPU: the C++ drop-in headers (integrators, interpolators, autodiff, regulators, fan-out
helpers, kernel math, the forwarding headers at the reference's include paths) compile for
sm_103a in a user translation unit -- the GPU test driver tests/cpp/test_integrators.cu, and a
small unit that includes every forwarding header by its reference path.  nvcc cross-compiles
without a GPU; nothing runs."""
import os
import subprocess

from diffrg_gb300 import build as B
from diffrg_gb300 import cppapi


def test_gpu_test_driver_compiles():
    out = cppapi.build_tests()
    assert os.path.exists(out)


def test_every_forwarding_header_compiles(tmp_path):
    compat = os.path.join(B.INCLUDE, "gbint", "compat")
    heads = sorted(os.path.relpath(os.path.join(d, f), compat) for d, _, fs in os.walk(compat) for f in fs
                   if f.endswith(".hh"))
    assert len(heads) >= 45
    src = tmp_path / "all_headers.cu"
    src.write_text("".join('#include <%s>\n' % h for h in heads) + '#include "gbint/kernel_math.hh"\n'
                   "int main() { return DiFfRG::powr<2>(1.0) == 1.0 ? 0 : 1; }\n")
    cmd = [B.nvcc(), "-std=c++17", "--expt-relaxed-constexpr", "-I", compat, "-I", B.INCLUDE] + B.ARCH + \
        ["-c", str(src), "-o", str(tmp_path / "all_headers.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
