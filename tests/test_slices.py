"""Cell-range slices of an integral area, checked on the host (no GPU).

The reference integrates each area's cells [min_calculation,
max_calculation) of the linearised (mu, nu, r) index
(cpu/evaluation_optimized.c:461-530; split_astronomy_parameters,
cpu/parameters.c:502-522).  tests/slice_harness.cpp compiles the library's
own slice and enumeration code (csrc/mwsep_internal.h) on the host and checks
cell for cell that its thread items and warp tiles visit exactly the cells the
reference's loop visits, for every slice of small grids and seeded rank splits
of larger ones.
"""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(REPO, "milkywayathome_client_gb300", "csrc")


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "vector_types.h")) else None


def test_enumeration_matches_reference_walk(tmp_path):
    inc = _cuda_include()
    if inc is None or not shutil.which("g++"):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = tmp_path / "slice_harness"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), "-I", CSRC, "-I", inc,
                        os.path.join(REPO, "tests", "slice_harness.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "slice harness: ok" in r.stdout
