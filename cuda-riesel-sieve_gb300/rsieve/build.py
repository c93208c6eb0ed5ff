"""Build librsieve_gb300.so (CUDA, sm_103a), the rsieve CLI and the oracle.

Everything is compiled in-tree into ``cuda-riesel-sieve_gb300/_build`` with
plain nvcc/g++ calls, translation units in parallel, one ``-gencode``.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # cuda-riesel-sieve_gb300/
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "librsieve_gb300.so")
CLI = os.path.join(BUILD, "rsieve")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]

CU_SOURCES = ["rs_kernels.cu", "rs_host.cu", "rs_static.cu", "rs_server.cu", "rs_selftest.cu"]
HEADERS = ["rs_arith.cuh", "rs_internal.h"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "rsieve.h")]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs)
        os.replace(tmp, LIB)
    cli_src = os.path.join(PKG, "cli", "rsieve_main.cpp")
    if force or _stale(CLI, [cli_src, LIB, os.path.join(INCLUDE, "rsieve.h")]):
        tmp = CLI + f".tmp{os.getpid()}"
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", tmp, "-L" + BUILD,
              "-lrsieve_gb300", "-Wl,-rpath,$ORIGIN"])
        os.replace(tmp, CLI)
    if verbose:
        print("built", LIB, CLI)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
