"""In-tree build of libmwsep_gb300.so (CUDA kernels + C ABI) for sm_103a.

Translation units are compiled in parallel and linked with nvcc; nothing is
installed outside the package directory.  The FP64 files are compiled with
``-fmad=false`` so no product or sum is fused (the reference CPU path
evaluates every operation separately); the compensated-FP32 file keeps FMA
contraction on.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_DIR = os.path.join(PKG_DIR, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libmwsep_gb300.so")
CLIENT_PATH = os.path.join(LIB_DIR, "mwsep_client")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]

# (source, extra nvcc flags)
UNITS = [
    ("mwsep_host.cu", ["-fmad=false"]),
    ("mwsep_geometry.cu", ["-fmad=false"]),
    ("mwsep_f64.cu", ["-fmad=false"]),
    ("mwsep_reduce.cu", ["-fmad=false"]),
    ("mwsep_f32.cu", ["-fmad=true"]),
    ("mwsep_peaks.cu", ["-fmad=true"]),
    ("mwsep_noalloc.cu", ["-fmad=false"]),
    ("mwsep_engine.cu", ["-fmad=false"]),
    ("mwsep_engine_f32.cu", ["-fmad=true"]),
    ("mwsep_engine_f64.cu", ["-fmad=false"]),
    ("mwsep_separation.cu", ["-fmad=false"]),
    ("mwsep_df.cu", ["-fmad=true"]),
    ("mwsep_io.cpp", []),
    ("mwsep_server.cpp", []),
    ("mwsep_optimise.cpp", []),
    ("mwsep_binary.cpp", []),
]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmwsep_gb300")


def _sources_newer_than(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit, extra, verbose, build_dir=BUILD_DIR):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(build_dir, unit + ".o")
    cmd = [nvcc(), "-c", src, "-o", obj, "-std=c++17", "-O3", "-lineinfo", *ARCH,
           "-I" + INCLUDE, "-I" + CSRC, "-Xcompiler", ",".join(HOST_FLAGS), *extra]
    if unit.endswith(".cpp"):
        cmd += ["-x", "c++"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {unit} failed:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False, extra_flags=(), lib_path: str = LIB_PATH,
          build_dir: str = BUILD_DIR) -> str:
    """Compile every translation unit and link the shared library.

    extra_flags / lib_path / build_dir build a variant elsewhere (for tuning
    experiments); the default is the in-tree library the package loads."""
    if not force and not extra_flags and not _sources_newer_than(lib_path):
        if lib_path == LIB_PATH and not os.path.exists(CLIENT_PATH):
            _build_client(verbose)
        return lib_path
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(os.path.dirname(lib_path), exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], list(u[1]) + list(extra_flags), verbose, build_dir), UNITS))
    tmp = lib_path + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-lpthread", "-ldl"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"linking libmwsep_gb300.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path)
    if lib_path == LIB_PATH:
        _build_client(verbose)
    return lib_path


def _build_client(verbose: bool) -> None:
    """The C command-line client (csrc/mwsep_client.c) linked against the library."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("a C compiler is required to build mwsep_client")
    cmd = [cc, "-O2", "-std=gnu99", "-I" + INCLUDE, os.path.join(CSRC, "mwsep_client.c"), "-L" + LIB_DIR,
           "-lmwsep_gb300", "-Wl,-rpath,$ORIGIN", "-o", CLIENT_PATH]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building mwsep_client failed:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
