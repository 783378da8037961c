"""In-tree build of the CUDA library ``libgbpf.so`` (sm_103a) from ``csrc/``.

Translation units are compiled in parallel (nvcc for the .cu files, g++ for the host
planner) and linked with nvcc; the result lands next to this file. Rebuilds only when a
source is newer than the library.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import tempfile

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(PKG), "csrc")
INCLUDE = os.path.join(os.path.dirname(os.path.dirname(PKG)), "include")
LIB = os.path.join(PKG, "libgbpf.so")

CU_SOURCES = ["gbpf.cu", "gbpf_kernels.cu", "islands.cu", "postproc.cu"]
CXX_SOURCES = ["plan.cpp"]
HEADERS = ["gbpf_device.h", "plan.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbpf.so")


def _sources():
    srcs = [os.path.join(CSRC, f) for f in CU_SOURCES + CXX_SOURCES + HEADERS]
    srcs.append(os.path.join(INCLUDE, "gbpf.h"))
    return srcs


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def compile_jobs(objdir: str):
    nv = nvcc()
    jobs = []
    for f in CU_SOURCES:
        out = os.path.join(objdir, f + ".o")
        jobs.append((out, [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
                           "-diag-suppress", "1444", "-c", os.path.join(CSRC, f), "-o", out]))
    for f in CXX_SOURCES:
        out = os.path.join(objdir, f + ".o")
        jobs.append((out, ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{INCLUDE}", "-c", os.path.join(CSRC, f), "-o",
                           out]))
    return jobs


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    with tempfile.TemporaryDirectory(prefix="gbpf_build_") as d:
        jobs = compile_jobs(d)
        procs = [(out, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
                 for out, cmd in jobs]
        errors = []
        for out, cmd, p in procs:
            log, _ = p.communicate()
            if p.returncode != 0:
                errors.append(" ".join(cmd) + "\n" + log)
            elif verbose and log.strip():
                print(log)
        if errors:
            raise RuntimeError("libgbpf build failed:\n" + "\n".join(errors))
        tmp = LIB + ".tmp"
        link = [nvcc(), *ARCH, "-shared", "-o", tmp] + [o for o, _ in jobs]
        p = subprocess.run(link, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("libgbpf link failed:\n" + " ".join(link) + "\n" + p.stdout + p.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
