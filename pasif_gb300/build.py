"""In-tree build of libpasif_gb300.so (sm_103a) and of the CPU oracle.

The library is compiled from pasif_gb300/csrc with nvcc for sm_103a only;
translation units are compiled in parallel and linked against the CUDA
runtime and NVRTC (the pattern-specialised kernels are compiled at run time).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpasif_gb300.so")
ROOT = os.path.dirname(HERE)
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(os.path.join(CUDA_HOME, "bin", "nvcc")) else "nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["generic_kernels.cu", "noalloc.cu"]
CPP_SOURCES = ["engine.cpp", "jit.cpp", "driver.cpp", "capi.cpp", "pattern.cpp", "pool.cpp"]
EMBEDDED = ["pk_args.h", "rk4_core.cuh"]


def _embed() -> str:
    """Write csrc/_embedded.h: the device headers as raw strings for NVRTC."""
    path = os.path.join(CSRC, "_embedded.h")
    parts = ["// generated by pasif_gb300/build.py: device headers for NVRTC\n#pragma once\n",
             "namespace pk_embedded {\n"]
    for name in EMBEDDED:
        with open(os.path.join(CSRC, name)) as f:
            text = f.read()
        assert ')PKRAW"' not in text
        ident = name.replace(".", "_")
        parts.append(f'static const char* const {ident} = R"PKRAW({text})PKRAW";\n')
    parts.append("}  // namespace pk_embedded\n")
    content = "".join(parts)
    old = open(path).read() if os.path.exists(path) else None
    if old != content:
        with open(path, "w") as f:
            f.write(content)
    return path


def _newest(paths) -> float:
    return max(os.path.getmtime(p) for p in paths)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    _embed()
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "pasif_gb300.h"),
                                                                os.path.abspath(__file__)]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(deps):
        return LIB
    inc = ["-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(OUT_DIR, src + ".o")
        jobs.append((obj, [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                           *inc, "-c", os.path.join(CSRC, src), "-o", obj]))
    for src in CPP_SOURCES:
        obj = os.path.join(OUT_DIR, src + ".o")
        jobs.append((obj, [NVCC, "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-Wall", *inc,
                           "-c", os.path.join(CSRC, src), "-o", obj]))
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        results = list(ex.map(lambda j: _run(j[1]), jobs))
    if verbose:
        for r in results:
            sys.stdout.write(r.stdout + r.stderr)
    libdir = os.path.join(CUDA_HOME, "lib64")
    tmp = LIB + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *[j[0] for j in jobs], "-lnvrtc", "-cudart", "shared",
          "-Xlinker", "-rpath," + libdir])
    os.replace(tmp, LIB)
    return LIB


def build_oracle() -> str:
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    make = shutil.which("make")
    odir = os.path.join(ROOT, "oracle")
    if make:
        _run([make, "-s", "-C", odir])
    else:  # pragma: no cover - make is part of the toolchain on both hosts
        os.makedirs(os.path.join(odir, "_build"), exist_ok=True)
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared", "-o",
              os.path.join(odir, "_build", "liboracle.so"), os.path.join(odir, "oracle.c"), "-lm"])
    return os.path.join(odir, "_build", "liboracle.so")


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
    print(build_oracle())
