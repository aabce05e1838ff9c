"""Build and load libtflows_krylov.so (the CUDA sm_103a kernels + C-ABI shim).

The library is compiled in-tree with nvcc (one -gencode for sm_103a, both
translation units in parallel) and loaded with ctypes.  There is no CPU
fallback: a missing or unloadable library raises.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "libtflows_krylov.so")
SOURCES = ("krylov.cu", "krylov_fma.cu", "shim.cu", "noalloc.cu", "tune.cu", "assembly.cu",
           "momentum.cu", "halo.cu", "meshio.cpp")
HEADERS = ("device_common.cuh", "krylov_kernels.cuh", "solver_entry.cuh", "internal.h",
           "assembly_internal.h")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fno-strict-aliasing", "-Xptxas", "-v" if os.environ.get(
                  "TFLOWS_PTXAS_VERBOSE") else "-O3"]

_lock = threading.Lock()
_lib = None


class NativeLibraryError(RuntimeError):
    pass


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise NativeLibraryError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(INCLUDE, "tflows_krylov.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library if a source is newer than the .so."""
    with _lock:
        if not force and not _stale():
            return LIB_PATH
        os.makedirs(BUILD, exist_ok=True)
        cc = nvcc()

        def compile_one(src):
            obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
            extra = os.environ.get("TFLOWS_NVCC_EXTRA", "").split()
            # the contracted build fuses multiply-adds; everything else keeps
            # the reference's separately rounded products and sums
            fmad = ["--fmad=true"] if src == "krylov_fma.cu" else ["--fmad=false"]
            cmd = [cc, *ARCH, *NVCC_FLAGS, *fmad, *extra, "-I", INCLUDE, "-c",
                   os.path.join(CSRC, src), "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise NativeLibraryError(f"nvcc failed for {src}:\n{r.stderr}")
            if verbose:
                print(r.stderr)
            return obj

        with ThreadPoolExecutor(len(SOURCES)) as ex:
            objs = list(ex.map(compile_one, SOURCES))
        tmp = LIB_PATH + ".tmp"
        cmd = [cc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise NativeLibraryError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB_PATH)
        return LIB_PATH


_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_VP = ctypes.c_void_p


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("tol_mode", ctypes.c_int),
                ("inner_rtol", ctypes.c_double), ("inner_maxiter", ctypes.c_int),
                ("max_refinements", ctypes.c_int), ("refine_restart", ctypes.c_int),
                ("ic_sweeps", ctypes.c_int),
                ("ic_bf16", ctypes.c_int), ("timeout_s", ctypes.c_double),
                ("block_size", ctypes.c_int), ("grid_blocks", ctypes.c_int),
                ("device", ctypes.c_int), ("inject_stall", ctypes.c_int),
                ("autotune", ctypes.c_int), ("rows_per_warp", ctypes.c_int),
                ("sweep_warps", ctypes.c_int), ("sweep_gate", ctypes.c_int),
                ("ic_tiled", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int),
                ("inner_iterations", ctypes.c_int), ("refinements", ctypes.c_int),
                ("ini_res", ctypes.c_double), ("fin_res", ctypes.c_double),
                ("seconds", ctypes.c_double), ("bytes", ctypes.c_double),
                ("block_size", ctypes.c_int), ("grid_blocks", ctypes.c_int),
                ("group_seconds", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Tuning(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_int), ("rows_per_warp", ctypes.c_int),
                ("grid_blocks", ctypes.c_int), ("sweep_warps", ctypes.c_int),
                ("candidates", ctypes.c_int), ("from_table", ctypes.c_int),
                ("us_per_iteration", ctypes.c_double),
                ("default_us_per_iteration", ctypes.c_double), ("sweep_gate", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchTuning(ctypes.Structure):
    _fields_ = [("block_size", ctypes.c_int), ("runs", ctypes.c_int),
                ("default_seconds", ctypes.c_double), ("tuned_seconds", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Mesh(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in ("NC", "NbC", "NS", "NSsh", "Nmat")]
                + [(n, ctypes.POINTER(ctypes.c_int)) for n in ("material", "SideC", "bcmark",
                                                              "CopyC")]
                + [(n, ctypes.POINTER(ctypes.c_double))
                   for n in ("xc", "yc", "zc", "volume", "delta", "WallDs", "Sx", "Sy", "Sz",
                             "Dx", "Dy", "Dz", "f", "xsp", "ysp", "zsp")])


class CalcpsFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("rho_n", "rho_o", "rho_oo", "u", "v", "w", "p",
                                                 "px", "py", "pz", "asave")]


NEWUVW_FIELDS = ("material", "rho_n", "rho_o", "rho_oo", "ui_n", "ui_o", "ui_oo", "duidi",
                 "duidj", "duidk", "dujdi", "dukdi", "dujdj", "dukdk", "pi", "source", "flux_u",
                 "flux", "ff", "scoef", "blend", "blend_tem", "urfc")


class NewuvwFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in NEWUVW_FIELDS]


class NewuvwParams(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in ("var", "nmat", "moin_problem", "convec", "cross",
                                             "diffus", "inert")]
                + [(n, ctypes.c_double) for n in ("visc", "dt", "urf")])


_SOLVER = [_I, _I, _I, _D, _I, _I, _I, _D, _D, _D, _I, _I, _D, _D, _D]
# tflows_exchange_fn / tflows_glosum_fn
EXCHANGE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, _D, ctypes.c_int)
GLOSUM_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, _D)

SIGNATURES = {
    "tflows_default_options": ([ctypes.POINTER(Options)], None),
    "tflows_set_options": ([ctypes.POINTER(Options)], ctypes.c_int),
    "tflows_cg": (_SOLVER, None),
    "tflows_bicg": (_SOLVER, None),
    "tflows_cgs": (_SOLVER, None),
    "tflows_prec1": ([_I, _I, _D, _I, _I, _I, _D, _I], None),
    "tflows_resid": ([_I, _I, _I, _D, _I, _I, _D, _D, _D], None),
    "tflows_last_status": ([], ctypes.c_int),
    "tflows_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "tflows_last_error": ([], ctypes.c_char_p),
    "tflows_last_result": ([ctypes.POINTER(Result)], None),
    "tflows_finalize": ([], None),
    "tflows_forget_topologies": ([], None),
    "tflows_set_halo": ([ctypes.c_int, ctypes.c_int, _I, _I, _I, EXCHANGE_FN, GLOSUM_FN, _VP],
                        ctypes.c_int),
    "tflows_clear_halo": ([], None),
    "tflows_solve_ex": ([ctypes.c_int, *_SOLVER, ctypes.POINTER(Options), ctypes.POINTER(Result)],
                        ctypes.c_int),
    "tflows_topology_create": ([ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_int, _VP, _VP, _VP,
                                ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "tflows_topology_destroy": ([_VP], None),
    "tflows_topology_transpose_map": ([_VP], _VP),
    "tflows_topology_patterns": ([_VP], ctypes.c_int),
    "tflows_solve_device": ([_VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Options), _VP, _VP,
                             _VP, _VP, ctypes.c_int, ctypes.c_double, _VP,
                             ctypes.POINTER(Result)], ctypes.c_int),
    "tflows_solve_batched_device": ([ctypes.c_int, _VP, _VP, _VP, ctypes.POINTER(Options), _VP, _VP,
                                     _VP, _VP, _VP, _VP, ctypes.POINTER(Result)], ctypes.c_int),
    "tflows_pattern_outer": ([_VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "tflows_ic_apply_device": ([_VP, ctypes.POINTER(Options), _VP, _VP, _VP, _VP,
                                ctypes.POINTER(Result)], ctypes.c_int),
    "tflows_spmv_device": ([_VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_int, _VP,
                            ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "tflows_plan_create": ([ctypes.POINTER(_VP), ctypes.c_int, _VP, _VP, _VP,
                            ctypes.POINTER(Options), _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "tflows_plan_launch": ([_VP, _VP], ctypes.c_int),
    "tflows_plan_results": ([_VP, ctypes.POINTER(Result)], ctypes.c_int),
    "tflows_plan_destroy": ([_VP], None),
    "tflows_plan_tuning": ([_VP, ctypes.POINTER(BatchTuning)], ctypes.c_int),
    "tflows_autotune": ([_VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Options), _VP, _VP, _VP,
                         ctypes.POINTER(Tuning)], ctypes.c_int),
    "tflows_autotune_clear": ([], None),
    "tflows_assembly_create": ([ctypes.POINTER(_VP), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int] + [_VP] * 12 + [ctypes.c_int], ctypes.c_int),
    "tflows_assembly_destroy": ([_VP], None),
    "tflows_calcps_assemble_device": ([_VP, ctypes.c_int, ctypes.c_double,
                                       ctypes.POINTER(CalcpsFields), _VP, _VP, _VP, _VP,
                                       ctypes.POINTER(ctypes.c_double), _VP,
                                       ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "tflows_newuvw_assemble_device": ([_VP, ctypes.POINTER(NewuvwParams),
                                       ctypes.POINTER(NewuvwFields), _VP, _VP, _VP, _VP, _VP,
                                       _VP, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "tflows_mesh_read": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.POINTER(Mesh))],
                         ctypes.c_int),
    "tflows_mesh_free": ([ctypes.POINTER(Mesh)], None),
    "tflows_topolm": ([ctypes.c_int, ctypes.c_int, _VP, _VP, _VP, _VP, _VP, _I], ctypes.c_int),
    "tflows_cg_noalloc": ([ctypes.c_int, _VP, _VP, _VP, _VP, _VP, _VP, _VP, ctypes.c_int,
                           ctypes.c_int, ctypes.c_double, _VP, _I, _D, _D], ctypes.c_int),
}


def header_symbols() -> list:
    """Function names declared in include/tflows_krylov.h."""
    import re
    text = open(os.path.join(INCLUDE, "tflows_krylov.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tflows_\w+)\s*\(", text)))


def load(path: str | None = None):
    """Load the shared library (building it first if needed) and bind every
    exported entry point.  Raises NativeLibraryError on failure."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
    p = path or os.environ.get("TFLOWS_LIB") or LIB_PATH
    if not os.path.exists(p):
        build()
    try:
        L = ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL)
    except OSError as e:
        raise NativeLibraryError(f"cannot load {p}: {e}") from e
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    with _lock:
        _lib = L
    return L
