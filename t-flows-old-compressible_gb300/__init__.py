"""GB300-native Krylov linear-solver core for T-FlowS (CG / BiCG / CGS + Prec1).

The solver path is libtflows_krylov.so (CUDA sm_103a kernels + a C ABI that
keeps the Fortran subroutine interfaces); this package builds and loads it,
mirrors the reference interface in Python (``cg``, ``bicg``, ``cgs``,
``prec1``, ``resid``), exposes the device-array ``Topology`` interface used
by the PyTorch binding, and generates the synthetic meshes of the benchmark.
"""
from . import mesh  # noqa: F401
from ._native import LIB_PATH, NativeLibraryError, build as build_library, header_symbols  # noqa: F401
from ._native import load as load_library  # noqa: F401
from .api import (  # noqa: F401
    BAD_INPUT, BICG, BICG_TRUE, BREAKDOWN, CG, CGS, CUDA_ERROR, FP64, FP64_FMA, HALO_ERROR, MIXED,
    NO_DEVICE, NONFINITE,
    NOT_CONVERGED, OK, TIMEOUT, TOL_ABSOLUTE, TOL_RELATIVE, UNSUPPORTED, SolveOutput, SolverError,
    Assembly, Plan, Topology, autotune_clear, bicg, cg, cgs, clear_halo, finalize, forget_topologies, last_error, last_result, last_status, options, prec1, resid,
    read_mesh, set_halo, set_options, solve_batched, solve_ex, solve_system, status_string, topolm,
)
