"""Build the CUDA extension (libmallocmc_gb300.so) for sm_103a, in-tree.

Each translation unit under csrc/ is compiled in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`, then linked into
one shared library next to this file. No torch extension machinery: the
library exports a plain C ABI (include/mallocmc_gb300.h) loaded with ctypes.
The same sources are also built with the device event counters compiled in
(-DMMC_DEVICE_STATS) into libmallocmc_gb300_stats.so, for tests and diagnosis.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_NAME = "libmallocmc_gb300.so"
LIB_PATH = os.path.join(PKG, LIB_NAME)
# the same library with the device event counters (MMC_DEVICE_STATS) compiled in
STATS_LIB_PATH = os.path.join(PKG, "libmallocmc_gb300_stats.so")
STATS_BUILD_DIR = os.path.join(BUILD_DIR, "stats")
EXAMPLES_PATH = os.path.join(PKG, "libmallocmc_examples.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["heap_capi.cu", "workloads.cu", "batch.cu", "serve.cu"]
EXAMPLE_SOURCES = ["cxx_examples.cu"]  # user-side code on the C++ API, linked against the library
TOOLS = ["verify_heap"]  # executables on the C++ API (csrc/<name>.cu -> mallocmc_gb300/<name>)


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC,
                   "--expt-relaxed-constexpr"]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    out = []
    for base in (CSRC, os.path.join(INCLUDE)):
        for dirpath, _, files in os.walk(base):
            out += [os.path.join(dirpath, f) for f in files if f.endswith((".h", ".cuh", ".hpp"))]
    return out


def build(verbose: bool = False, ptxas_verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    hdrs = _headers()
    objs, jobs = [], []
    ex_objs = []
    for src in EXAMPLE_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        ex_objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + _flags() + ["-c", s, "-o", o])
    tool_objs = []
    for name in TOOLS:
        s = os.path.join(CSRC, name + ".cu")
        o = os.path.join(BUILD_DIR, name + ".o")
        tool_objs.append((name, o))
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + _flags() + ["-c", s, "-o", o])
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            cmd = [nvcc()] + _flags() + (["-Xptxas", "-v"] if ptxas_verbose else []) + ["-c", s, "-o", o]
            jobs.append(cmd)
    os.makedirs(STATS_BUILD_DIR, exist_ok=True)
    stats_objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(STATS_BUILD_DIR, src.replace(".cu", ".o"))
        stats_objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + _flags() + ["-DMMC_DEVICE_STATS", "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_verbose:
                sys.stdout.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if _stale(LIB_PATH, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB_PATH] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if _stale(STATS_LIB_PATH, stats_objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", STATS_LIB_PATH] + stats_objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if _stale(EXAMPLES_PATH, ex_objs + [LIB_PATH]):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", EXAMPLES_PATH] + ex_objs + \
            ["-L" + PKG, "-lmallocmc_gb300", "-Xlinker", "-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    for name, o in tool_objs:
        exe = os.path.join(PKG, name)
        if _stale(exe, [o, LIB_PATH]):
            cmd = [nvcc()] + ARCH + ["-cudart", "static", "-o", exe, o, "-L" + PKG, "-lmallocmc_gb300",
                                     "-Xlinker", "-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True, ptxas_verbose="-v" in sys.argv))
