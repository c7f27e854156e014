"""The integrator classes the reference's code generator writes into a generated flow, mapped
onto this library's drop-in classes.

DiFfRG's Mathematica code generator picks the integrator class of every generated kernel from
the kernel's specification: ``Type`` ("Quadrature", "CartesianQuadrature", "QMC", "Constant"
at T = 0; "Quadraturex0" / "Quadratureq0" at finite T), ``Device`` ("CPU", "TBB", "GPU"), the
dimension ``d``, the number of ``Angles`` and the compute type ``ctype``
(Mathematica/DiFfRG/CodeTools.m: ``DeviceChoice`` :392-394, ``MakeIntegratorTypes`` :1167-1215,
``MakeKernelIntegratorFiniteTx0`` :1487-1510, ``MakeKernelIntegratorFiniteTq0`` :1684-1707), and
writes ``std::unique_ptr<DiFfRG::...>`` members constructed as
``(quadrature_provider, grid_sizes, x_extent, json)`` (:1333-1345).  The drop-in headers
(``include/gbint/compat``) define every class name that choice can produce, so generated code
compiles unchanged; ``integrator_types`` restates the choice (the same names, in this
repository's code) and ``family`` names the GB300 family each class runs on.
``tests/test_codegen_types.py`` compiles every name against the drop-in headers.
"""
from __future__ import annotations

from dataclasses import dataclass

DEVICE_SUFFIX = {"CPU": "TBB", "TBB": "TBB", "GPU": "GPU"}
TYPES_T0 = ("QMC", "Constant", "Quadrature", "CartesianQuadrature")
TYPES_FINITE_T = ("Quadraturex0", "Quadratureq0")


class CodegenError(ValueError):
    """A kernel specification the reference's generator rejects (it prints and aborts)."""


@dataclass(frozen=True)
class KernelSpec:
    name: str
    type: str = "Quadrature"
    device: str = "GPU"
    d: int = 4
    angles: int = 0
    ctype: str = "double"
    ad: bool = False


def integrator_types(k: KernelSpec) -> tuple[str, str]:
    """(integrator, integrator_AD): the C++ types the generated ``<Name>.hh`` declares for the
    kernel; the AD type is used when ``k.ad`` is set."""
    kern = f"{k.name}_kernel<__REGULATOR__>"
    if k.type in TYPES_FINITE_T:
        dev = _device(k.device)
        base = "FiniteTx0" if k.type == "Quadraturex0" else "FiniteTq0"
        if k.angles == 0:
            cls, lead = f"Integrator{base}{dev}", f"{k.d}, "
        elif k.angles == 1:
            cls, lead = f"IntegratorAngle{base}{dev}", f"{k.d}, "
        elif k.angles == 2:
            if k.d != 4:
                raise CodegenError("Inconsistent dimensions!")
            cls, lead = f"Integrator4D{base}{dev}", ""
        else:
            raise CodegenError("finite-T kernels have 0, 1 or 2 angles")
        return _pair(cls, lead, k.ctype, kern)
    if k.type not in TYPES_T0:
        raise CodegenError("Unknown integration type " + k.type + "!")
    if k.type == "QMC":
        suffix = "QMC"
    elif k.type == "Constant":
        if k.angles != 0:
            raise CodegenError("Constant integrator cannot have angles!")
        suffix = "Constant"
    elif k.type == "Quadrature":
        suffix = _device(k.device)
    else:
        if k.angles != 0:
            raise CodegenError("Cartesian integrator cannot have angles!")
        suffix = "Cartesian" + _device(k.device)
    if k.type == "CartesianQuadrature":
        return _pair(f"Integrator{k.d}D{suffix}", "", k.ctype, kern)
    if k.angles == 0:
        return _pair(f"Integrator{suffix}", f"{k.d}, ", k.ctype, kern)
    if k.angles == 1:
        return _pair(f"IntegratorAngle{suffix}", f"{k.d}, ", k.ctype, kern)
    if k.angles == 2:
        if k.d not in (3, 4):
            raise CodegenError("Inconsistent dimensions!")
        cls = f"Integrator3D{suffix}" if k.d == 3 else f"Integrator4D2Ang{suffix}"
        return _pair(cls, "", k.ctype, kern)
    if k.angles == 3:
        if k.d != 4:
            raise CodegenError("Inconsistent dimensions!")
        return _pair(f"Integrator4D{suffix}", "", k.ctype, kern)
    raise CodegenError("T = 0 kernel cannot have > 3 angles!")


def grid_size_count(k: KernelSpec) -> int:
    """Length of the ``std::array<uint, N>`` of grid sizes the generated constructor takes
    (CodeTools.m :1228-1231: angles + 1, or d for Cartesian kernels; :1541 angles + 2 for the x0
    kernels, whose last order is the tail's; :1720 angles + 1 for the q0 kernels)."""
    if k.type == "CartesianQuadrature":
        return k.d
    return k.angles + 2 if k.type == "Quadraturex0" else k.angles + 1


def constructor_arguments(k: KernelSpec) -> str:
    """The arguments the generated wrapper constructs the integrator with (CodeTools.m :1336,
    :1618, :1811)."""
    if k.type == "Quadraturex0":
        return "quadrature_provider, grid_sizes, x_extent, x0_extent, x0_summands, json"
    return "quadrature_provider, grid_sizes, x_extent, json"


# The GB300 family each drop-in class runs on (include/gbint/device/families.cuh; the C ABI's
# families in include/gbint.h).  The reference's CPU (TBB) classes run on the same families.
_FAMILY = {
    "Integrator": "F1D (radial)", "IntegratorAngle": "FAngle", "Integrator3D": "F3D",
    "Integrator4D2Ang": "F4D2Ang", "Integrator4D": "F4D", "IntegratorCartesian": "FCart",
    "IntegratorConstant": "constant (no grid)", "IntegratorQMC": "QMC lattice (1 variable)",
    "IntegratorAngleQMC": "QMC lattice (2 variables)", "Integrator4DQMC": "QMC lattice (4 variables)",
    "IntegratorFiniteTx0": "FTx0<d, 0>", "IntegratorAngleFiniteTx0": "FTx0<d, 1>",
    "Integrator4DFiniteTx0": "FTx0<4, 2>", "IntegratorFiniteTq0": "FTq0<d, 0>",
    "IntegratorAngleFiniteTq0": "FTq0<d, 1>", "Integrator4DFiniteTq0": "FTq0<4, 2>",
}


def family(integrator: str) -> str:
    """The GB300 family of a generated integrator type, e.g.
    ``family("DiFfRG::IntegratorAngleGPU<4, double, ZA_kernel<__REGULATOR__>>") == "FAngle"``."""
    cls = integrator.split("<", 1)[0].replace("DiFfRG::", "")
    for suf in ("GPU", "TBB"):
        if cls.endswith(suf):
            cls = cls[: -len(suf)]
    if cls.endswith("DCartesian"):
        return _FAMILY["IntegratorCartesian"] + cls[len("Integrator"):-len("DCartesian")]
    if cls not in _FAMILY:
        raise CodegenError("not an integrator the generator writes: " + integrator)
    return _FAMILY[cls]


def all_specs(name: str = "K"):
    """Every specification the generator accepts (dimensions 1..4, both compute types): the
    list the compile test instantiates."""
    out = []
    for ctype in ("double", "float"):
        for dev in ("CPU", "TBB", "GPU"):
            for t in ("Quadrature", "QMC"):
                if t == "QMC" and dev != "GPU":
                    continue  # the QMC choice ignores the device
                for ang in range(4):
                    for d in range(1, 5):
                        if ang == 2 and d not in (3, 4):
                            continue
                        if ang == 3 and d != 4:
                            continue
                        if ang >= 1 and d < 2:
                            continue
                        if t == "QMC" and not _qmc_exists(ang, d):
                            continue
                        out.append(KernelSpec(name, t, dev, d, ang, ctype))
            for d in (1, 2, 3):
                out.append(KernelSpec(name, "CartesianQuadrature", dev, d, 0, ctype))
            for t in TYPES_FINITE_T:
                for ang in range(3):
                    for d in (1, 2, 3, 4):
                        if ang == 2 and d != 4:
                            continue
                        if ang >= 1 and d < 2:
                            continue
                        out.append(KernelSpec(name, t, dev, d, ang, ctype))
        for d in (1, 2, 3, 4):
            out.append(KernelSpec(name, "Constant", "GPU", d, 0, ctype))
    return out


def _qmc_exists(angles: int, d: int) -> bool:
    """The reference ships IntegratorQMC<d>, IntegratorAngleQMC<d> and Integrator4DQMC only
    (DiFfRG/include/DiFfRG/physics/integration/integrator{,_angle,_4D}_qmc.hh); the generator's
    other QMC names (3D, 4D2Ang) have no class there either."""
    return angles in (0, 1) or (angles == 3 and d == 4)


def _device(dev: str) -> str:
    if dev not in DEVICE_SUFFIX:
        raise CodegenError("Unknown device " + dev)
    return DEVICE_SUFFIX[dev]


def _pair(cls: str, lead: str, ctype: str, kern: str) -> tuple[str, str]:
    return (f"DiFfRG::{cls}<{lead}{ctype}, {kern}>", f"DiFfRG::{cls}<{lead}autodiff::real, {kern}>")
