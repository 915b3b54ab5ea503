"""Builds the native libraries of the package in-tree.

* ``lib/libpeec_mesh.so``  -- host-only voxel mesher (g++, OpenMP).
* ``lib/libpeec_gb300.so`` -- the sm_103a CUDA kernels and the C ABI declared in
  ``include/peec_gb300.h`` (nvcc, one ``-gencode`` for compute_103a/sm_103a).

Translation units compile in parallel; objects go to ``_build/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BUILD = ROOT / "_build" / "solver_gb300"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC)]

MESH_SOURCES = ["mesher.cpp"]
CUDA_SOURCES = ["ctx.cu", "fftconv.cu", "fftconv_f32.cu", "fftconv_f64.cu", "fftconv_ff.cu",
                "krylov.cu", "sparse.cu", "fill.cu", "adjoint.cu", "refactor.cu",
                "mesher_gpu.cu", "dense.cu"]
# the fill keeps the reference's scalar rounding: no FMA contraction
FILE_FLAGS = {"fill.cu": ["-fmad=false"]}
CUDA_HEADERS = ["common.cuh", "fft.cuh", "fft_reg.cuh", "fftconv_impl.cuh",
                "ctx.hpp"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build solver_gb300")


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        h.update(Path(p).read_bytes())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    h.update(repr(sorted(FILE_FLAGS.items())).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build_mesh(force: bool = False) -> Path:
    LIBDIR.mkdir(parents=True, exist_ok=True)
    out = LIBDIR / "libpeec_mesh.so"
    srcs = [CSRC / s for s in MESH_SOURCES]
    stamp = LIBDIR / ".mesh.stamp"
    dig = _digest(srcs)
    if out.exists() and stamp.exists() and stamp.read_text() == dig and not force:
        return out
    cxx = shutil.which("g++") or "g++"
    _run([cxx, "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-shared", "-o", str(out)] +
         [str(s) for s in srcs])
    stamp.write_text(dig)
    return out


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    LIBDIR.mkdir(parents=True, exist_ok=True)
    BUILD.mkdir(parents=True, exist_ok=True)
    out = LIBDIR / "libpeec_gb300.so"
    srcs = [CSRC / s for s in CUDA_SOURCES]
    hdrs = [CSRC / h for h in CUDA_HEADERS if (CSRC / h).exists()] + [INCLUDE / "peec_gb300.h"]
    stamp = LIBDIR / ".cuda.stamp"
    dig = _digest(srcs + hdrs)
    if out.exists() and stamp.exists() and stamp.read_text() == dig and not force:
        return out
    nvcc = nvcc_path()

    def compile_one(src: Path) -> str:
        obj = BUILD / (src.stem + ".o")
        cmd = ([nvcc] + ARCH + NVCC_FLAGS + FILE_FLAGS.get(src.name, []) +
               ["-Xptxas", "-v", "-c", str(src), "-o", str(obj)])
        return _run(cmd)

    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        logs = list(ex.map(compile_one, srcs))
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    (BUILD / "ptxas.log").write_text("\n".join(logs))
    objs = [str(BUILD / (s.stem + ".o")) for s in srcs]
    _run([nvcc] + ARCH + ["-shared", "-o", str(out)] + objs + ["-lcudart"])
    stamp.write_text(dig)
    return out


def build_all(force: bool = False, verbose: bool = False):
    return build_mesh(force), build_cuda(force, verbose)


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv, verbose="-v" in sys.argv))
