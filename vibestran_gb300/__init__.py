"""vibestran_gb300 — GB300-native (sm_103a) SOL 101 CHEXA8 backend for vibestran.

The compute path is ``libvsgb.so`` (hand-written CUDA, C ABI in include/vsgb.h);
this package holds its build script, the ctypes host mirror of the reference's
SolverBackend interface and a synthetic-model generator.
"""
from .backend import (  # noqa: F401
    EAS, FP64, MIXED, SRI, ChexaAssembler, CsrData, Gb300MixedPcgSolverBackend,
    Gb300PcgSolverBackend, SolverError, apply_forces, build_dof_map, load_library)
