"""diffrg_gb300 -- GB300-native engine for DiFfRG's momentum-loop integrals.

The compute path is libgbint.so (hand-written sm_103a CUDA behind a C ABI, include/gbint.h);
this package holds its Python host side, the in-tree build and the benchmark workloads.
"""
from .capi import FAM, IG, PREC, GbError  # noqa: F401

__all__ = ["FAM", "IG", "PREC", "GbError"]
