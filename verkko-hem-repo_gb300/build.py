"""Builds libglgpu.so (the C-ABI library) for sm_103a, in-tree.

Host C++ (plan, mesher, material parameters) is compiled with g++; the CUDA
translation units with nvcc ``-gencode arch=compute_103a,code=sm_103a``.  All
objects compile in parallel; outputs go to ``<package>/_build`` and the library to
``<package>/lib/libglgpu.so``.  Nothing is installed outside the tree.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libglgpu.so")
DRIVER = os.path.join(LIBDIR, "femgl_gb300")
INCLUDE = os.path.join(ROOT, "include")

CU_SOURCES = ["kernels_asm.cu", "kernels_la.cu", "kernels_mg.cu", "kernels_mf.cu", "kernels_est.cu", "glgpu.cu", "noalloc.cu",
              "mlp.cu"]
CC_SOURCES = ["host_util.cc", "plan.cc", "mg.cc", "kelly.cc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile everything that is out of date and return the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(INCLUDE, "glgpu.h"))
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s, *headers]):
            jobs.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I",
                         CSRC, "-c", s, "-o", o])
    for src in CC_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s, *headers]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-I", INCLUDE, "-I", CSRC, "-c", s, "-o", o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((j, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + o for j, o in failed)
        raise RuntimeError("glgpu build failed:\n" + msg)
    if force or jobs or not os.path.exists(LIB):
        cuda_lib = os.path.join(_cuda_home(), "lib64")
        link = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-Xcompiler", "-fopenmp", "-lgomp", "-L", cuda_lib,
                "-lcudart"]
        subprocess.run(link, check=True, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        os.replace(LIB + ".tmp", LIB)
    drv_src = os.path.join(CSRC, "femgl_main.cc")
    if os.path.exists(drv_src) and (force or not _newer(DRIVER, [drv_src, LIB])):
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, drv_src, "-o", DRIVER, "-L", LIBDIR, "-lglgpu",
                        "-Wl,-rpath,$ORIGIN"], check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
