"""A C program built with gcc calls the Fortran-facing entry points with the
reference's array layout: 1-based CSR from TopolM, x passed from x(-NB),
boundary values and x(0) that must stay untouched (c_caller/
fortran_layout_caller.c).  On the CPU the program must build, link against
the in-tree library and exit with the library's no-device status; on a GPU
its checks (Prec1 and Resid bit for bit against the restated loops, CG to
the tolerance) must pass."""
import os
import shutil
import subprocess

import pytest

from conftest import tflows

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _build(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    tflows.load_library()  # builds the library when it is missing or stale
    lib_dir = os.path.dirname(tflows._native.LIB_PATH)
    rpaths = [lib_dir]
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")
    if os.path.isdir(cuda_lib):
        rpaths.append(cuda_lib)
    exe = str(tmp_path / "fortran_layout_caller")
    cmd = [cc, "-O2", "-ffp-contract=off", "-std=c11", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "c_caller",
                                                             "fortran_layout_caller.c"),
           "-L", lib_dir, "-ltflows_krylov", *[f"-Wl,-rpath,{p}" for p in rpaths], "-lm",
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_caller_builds_and_reports_no_device(tmp_path):
    import torch
    exe = _build(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present: the GPU test runs the checks")
    r = subprocess.run([exe, "6", "5", "4"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 3, r.stdout + r.stderr
    assert "no CUDA device" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [("12", "10", "9"), ("31", "7", "5")])
def test_c_caller_fortran_layout_on_gpu(tmp_path, dims):
    exe = _build(tmp_path)
    r = subprocess.run([exe, *dims], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
