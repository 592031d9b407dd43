"""Builds the native library ``siml_gb300/libsiml_gb300.so`` in-tree.

CUDA sources are compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``); host C++ sources with the system g++.
Translation units compile in parallel and the objects are linked with nvcc
(static CUDA runtime), so the library needs nothing but the driver at run
time.  Usage: ``python -m siml_gb300.build`` or ``siml_gb300.build.build()``.
"""
from __future__ import annotations

import concurrent.futures as _cf
import os
import platform
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
OBJ_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libsiml_gb300.so")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if os.path.exists(cand):
        return cand
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")
    return found


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles every CUDA and C++ source of the package; returns the .so path."""
    nvcc = _nvcc()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    os.makedirs(OBJ_DIR, exist_ok=True)
    # objects built on another machine type are discarded
    stamp = os.path.join(OBJ_DIR, "MACHINE")
    machine = platform.machine()
    old = open(stamp).read().strip() if os.path.exists(stamp) else ""
    if old != machine:
        for f in os.listdir(OBJ_DIR):
            os.remove(os.path.join(OBJ_DIR, f))
        if os.path.exists(LIB_PATH):
            os.remove(LIB_PATH)
        with open(stamp, "w") as fh:
            fh.write(machine)
    cu, cpp = _sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "siml_gb300.h"))
    jobs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ_DIR, f + ".o")
        cmd = [nvcc, GENCODE, "-O3", "-lineinfo", "-std=c++17", "--fmad=false",
               "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
               "-c", src, "-o", obj]
        if ptxas_info:
            cmd.insert(3, "-Xptxas=-v")
        jobs.append((obj, [src] + headers, cmd))
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ_DIR, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
               "-I", INCLUDE, "-I", CSRC, "-I", cuda_inc, "-c", src, "-o", obj]
        jobs.append((obj, [src] + headers, cmd))

    def run(job):
        obj, deps, cmd = job
        if not ptxas_info and not _newer(obj, deps):
            return obj, ""
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        return obj, r.stdout + r.stderr

    with _cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        results = list(ex.map(run, jobs))
    if verbose or ptxas_info:
        for obj, out in results:
            if out.strip():
                print(os.path.basename(obj), out, file=sys.stderr)
    objs = [o for o, _ in results]
    if _newer(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc, GENCODE, "-shared", "-o", tmp] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
