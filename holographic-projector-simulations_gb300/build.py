"""Build the native library (libholo.so) and the `holo` CLI in-tree with nvcc.

Every translation unit under csrc/ is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
``libholo.so`` beside this file; ``holo`` (the reference-compatible command
line) links against it with an $ORIGIN rpath.  Objects go to ``_build/``.
A unit is recompiled only when its source or a shared header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(REPO, "include")
LIB = os.path.join(HERE, "libholo.so")
CLI = os.path.join(HERE, "holo")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_UNITS = ["abi.cu", "batch.cu", "epilogue.cu", "kernel_fp64.cu", "kernel_split.cu",
             "kernel_tc.cu", "noalloc.cu", "probe.cu", "tiler.cu"]
CLI_UNITS = ["cli.cpp", "io.cpp", "gen.cu"]
HEADERS = ["internal.cuh", "ptx.cuh", "split_frame.cuh", "io.h", "gen.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libholo")


def _newer(src: list[str], dst: str) -> bool:
    if not os.path.exists(dst):
        return True
    t = os.path.getmtime(dst)
    return any(os.path.exists(s) and os.path.getmtime(s) > t for s in src)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n"
                           f"{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile libholo.so and the holo CLI; return the library path."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "holo.h")]
    # host code rounds every product and sum on its own (no fused multiply-add), on
    # x86-64 and aarch64 alike: the CLI's plane geometry then equals the reference's
    common = ["-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]
    jobs = []
    objs = []
    for unit in LIB_UNITS + CLI_UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, os.path.splitext(unit)[0] + ".o")
        if unit in LIB_UNITS:
            objs.append(obj)
        if force or _newer([src] + headers, obj):
            flags = common + (["-x", "cu"] if unit.endswith(".cu") else ["-x", "c++"])
            jobs.append([cc, *flags, "-c", src, "-o", obj])
    workers = max(1, min(len(jobs), os.cpu_count() or 1))
    if jobs:
        with ThreadPoolExecutor(workers) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or _newer(objs, LIB):
        _run([cc, "-shared", *ARCH, "-o", LIB, *objs], verbose)
    cli_objs = [os.path.join(BUILD, os.path.splitext(u)[0] + ".o") for u in CLI_UNITS]
    if force or _newer(cli_objs + [LIB], CLI):
        _run([cc, *ARCH, "-o", CLI, *cli_objs, f"-L{HERE}", "-lholo", "-lcurand",
              "-Xlinker", "-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
