"""CPU: the code generator's integrator choice mapped onto the drop-in classes (row f3).

* ``diffrg_gb300.codegen.integrator_types`` restates which class DiFfRG's Mathematica generator
  writes for a kernel specification (CodeTools.m MakeIntegratorTypes and its finite-T twins);
  every name it can produce, for every accepted specification and both compute types, compiles
  against the drop-in headers as the generated wrapper uses it: constructed from
  (QuadratureProvider&, std::array<uint, N>, x_extent, JSONValue), with get<>/request<> calls
  (one translation unit, nvcc for sm_103a, nothing runs);
* the rejections the generator prints (angles on a Constant or Cartesian kernel, inconsistent
  dimensions, unknown types) are rejected;
* when a DiFfRG checkout is present ($GBINT_REFERENCE_DIR, or 'reference' beside this
  repository), every integrator member of the generated example flows is one the restated choice
  produces (read at test time, nothing copied).
"""
import os
import re
import subprocess

import pytest

from diffrg_gb300 import build as B
from diffrg_gb300 import codegen as CG

HERE = os.path.dirname(os.path.abspath(__file__))
COMPAT = os.path.join(B.INCLUDE, "gbint", "compat")


def test_choice_examples():
    assert CG.integrator_types(CG.KernelSpec("ZA", "Quadrature", "GPU", 4, 1))[0] == \
        "DiFfRG::IntegratorAngleGPU<4, double, ZA_kernel<__REGULATOR__>>"
    assert CG.integrator_types(CG.KernelSpec("ZA3", "Quadrature", "GPU", 4, 2))[0] == \
        "DiFfRG::Integrator4D2AngGPU<double, ZA3_kernel<__REGULATOR__>>"
    assert CG.integrator_types(CG.KernelSpec("V", "Quadrature", "CPU", 3, 0, ad=True))[1] == \
        "DiFfRG::IntegratorTBB<3, autodiff::real, V_kernel<__REGULATOR__>>"
    assert CG.integrator_types(CG.KernelSpec("e", "Quadratureq0", "TBB", 4, 1))[0] == \
        "DiFfRG::IntegratorAngleFiniteTq0TBB<4, double, e_kernel<__REGULATOR__>>"
    assert CG.integrator_types(CG.KernelSpec("c", "CartesianQuadrature", "GPU", 2, 0))[0] == \
        "DiFfRG::Integrator2DCartesianGPU<double, c_kernel<__REGULATOR__>>"
    assert CG.integrator_types(CG.KernelSpec("q", "QMC", "GPU", 4, 3))[0] == \
        "DiFfRG::Integrator4DQMC<double, q_kernel<__REGULATOR__>>"
    assert CG.family("DiFfRG::IntegratorAngleGPU<4, double, ZA_kernel<__REGULATOR__>>") == "FAngle"
    assert CG.family("DiFfRG::Integrator2DCartesianTBB<double, c_kernel<__REGULATOR__>>") == "FCart2"
    assert CG.grid_size_count(CG.KernelSpec("x", "Quadrature", "GPU", 4, 3)) == 4
    assert CG.grid_size_count(CG.KernelSpec("x", "CartesianQuadrature", "GPU", 3, 0)) == 3
    assert CG.grid_size_count(CG.KernelSpec("x", "Quadraturex0", "GPU", 4, 1)) == 3
    assert "x0_summands" in CG.constructor_arguments(CG.KernelSpec("x", "Quadraturex0", "GPU", 4, 1))


@pytest.mark.parametrize("spec", [
    CG.KernelSpec("a", "Constant", "GPU", 4, 1), CG.KernelSpec("b", "CartesianQuadrature", "GPU", 2, 1),
    CG.KernelSpec("c", "Quadrature", "GPU", 2, 2), CG.KernelSpec("d", "Quadrature", "GPU", 3, 3),
    CG.KernelSpec("e", "Quadrature", "GPU", 4, 4), CG.KernelSpec("f", "Quadraturex0", "GPU", 3, 2),
    CG.KernelSpec("g", "Sparse", "GPU", 4, 0), CG.KernelSpec("h", "Quadrature", "FPGA", 4, 0)])
def test_generator_rejections(spec):
    with pytest.raises(CG.CodegenError):
        CG.integrator_types(spec)


def _translation_unit(specs):
    lines = ['#include <DiFfRG/physics/integration.hh>', '#include <DiFfRG/physics/integration_finiteT.hh>',
             '#include <array>', '#include <type_traits>', '',
             'struct Reg {};', '#define __REGULATOR__ Reg',
             'template <typename REG> struct K_kernel {',
             '  template <typename... T> static __host__ __device__ double kernel(const T &...) { return 1.0; }',
             '  template <typename... T> static __host__ __device__ double constant(const T &...) { return 0.0; }',
             '};',
             'template <class I, class CT, std::size_t N, bool X0> constexpr bool generated_use()',
             '{',
             '  if constexpr (X0)',
             '    static_assert(std::is_constructible_v<I, DiFfRG::QuadratureProvider &, std::array<uint, N>, CT, CT,',
             '                                          uint, const DiFfRG::JSONValue &>);',
             '  else',
             '    static_assert(std::is_constructible_v<I, DiFfRG::QuadratureProvider &, std::array<uint, N>, CT,',
             '                                          const DiFfRG::JSONValue &>);',
             '  return requires(I &i, CT k) {',
             '    i.get(k, 1.0, 2.0);',
             '    i.request(k, 1.0, 2.0);',
             '  };',
             '}', '']
    seen = set()
    for s in specs:
        for which, t in enumerate(CG.integrator_types(s)):
            if which == 1 and s.ctype != "double":
                continue  # the generator pairs autodiff::real with double kernels
            if t in seen:
                continue
            seen.add(t)
            lines.append("static_assert(generated_use<%s, %s, %d, %s>(), \"%s\");" % (
                t, s.ctype, CG.grid_size_count(s), "true" if s.type == "Quadraturex0" else "false", t))
    return "\n".join(lines) + "\n", seen


def test_every_generated_name_compiles(tmp_path):
    src, names = _translation_unit(CG.all_specs("K"))
    assert len(names) > 150
    f = tmp_path / "codegen_types.cu"
    f.write_text(src)
    cmd = [B.nvcc(), "-std=c++20", "--expt-relaxed-constexpr", "-I", COMPAT, "-I", B.INCLUDE] + B.ARCH + \
        ["-c", str(f), "-o", str(tmp_path / "codegen_types.o")]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-4000:]


def _reference_dir():
    for d in (os.environ.get("GBINT_REFERENCE_DIR"), os.path.join(os.path.dirname(HERE), "..", "reference")):
        if d and os.path.isdir(os.path.join(d, "Examples")):
            return d
    return None


def test_generated_examples_are_reproduced():
    ref = _reference_dir()
    if ref is None:
        pytest.skip("no DiFfRG checkout (set GBINT_REFERENCE_DIR)")
    produced = set()
    for s in CG.all_specs("X"):
        for t in CG.integrator_types(s):
            produced.add(t)
    pat = re.compile(r"std::unique_ptr<(DiFfRG::[A-Za-z0-9]+<[^;]*>)>\s+integrator(?:_AD)?;")
    found = 0
    for root, _, files in os.walk(os.path.join(ref, "Examples")):
        for fn in files:
            if not fn.endswith(".hh") or "flows" not in root:
                continue
            for t in pat.findall(open(os.path.join(root, fn), errors="replace").read()):
                found += 1
                generic = re.sub(r"[A-Za-z0-9_]+_kernel<__REGULATOR__>", "X_kernel<__REGULATOR__>", t)
                assert generic in produced, (fn, t)
    assert found >= 28
