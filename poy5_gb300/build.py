"""Build libpoyalgn.so (sm_103a) in-tree: ``python -m poy5_gb300.build``.

Translation units are compiled in parallel with nvcc and linked into
``poy5_gb300/libpoyalgn.so``; nothing is installed elsewhere.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "libpoyalgn.so")
BUILD_DIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
UNITS = ["pa_kernels.cu", "pa_cost.cu", "pa_capi.cu", "pa_driver.cu", "pa_server.cu",
         "pa_newkk.cu", "pa_peak.cu", "pa_ukk3.cu", "pa_tables.cpp"]
HEADERS = ["pa_core.cuh", "pa_kernels.h", "pa_tables.h", "pa_runtime.h", "pa_cost.h",
           "pa_newkk.cuh", "pa_ukk3.cuh"]


def _deps():
    return ([os.path.join(CSRC, u) for u in UNITS + HEADERS] +
            [os.path.join(ROOT, "include", "poyalgn.h")])


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str, verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD_DIR, unit + ".o")
    cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-Werror=return-type",
           "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
    if unit.endswith(".cu") and verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA library if any source is newer than the .so."""
    if not force and not _stale(OUT, _deps()):
        return OUT
    os.makedirs(BUILD_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u, verbose), UNITS))
    tmp = OUT + ".tmp"
    res = subprocess.run([NVCC, *ARCH, "-shared", "-o", tmp, *objs],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
