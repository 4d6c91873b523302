"""Builds libvedas_gb300.so in-tree for sm_103a (nvcc, one -gencode)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvedas_gb300.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["vg_sort.cu", "vg_index.cu", "vg_relops.cu", "vg_batch.cu", "vg_noalloc.cu", "vg_ingest.cu", "vg_selfcheck.cu"]
CPP_SOURCES = ["vg_ctx.cpp", "vg_storage.cpp", "vg_capi.cpp", "compat/vedas_compat.cpp",
               "vg_batch_host.cpp", "vg_serve.cpp"]

COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + CSRC,
          "-I" + os.path.join(os.path.dirname(HERE), "include")]


def _sources():
    cu = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    cpp = [s for s in CPP_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    return cu, cpp


def _compile(src: str, extra: list) -> str:
    obj = os.path.join(OUT_DIR, src.replace("/", "_") + ".o")
    cmd = [NVCC] + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _stale(objs_from: list) -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in objs_from]
    for root, _, files in os.walk(CSRC):
        for f in files:
            if f.endswith((".h", ".cuh")):
                deps.append(os.path.join(root, f))
    deps.append(os.path.join(os.path.dirname(HERE), "include", "vedas_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    cu, cpp = _sources()
    if not force and not _stale(cu + cpp):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs = [(s, [GENCODE, "-lineinfo"]) for s in cu] + [(s, []) for s in cpp]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda a: _compile(*a), jobs))
    tmp = LIB + ".tmp"
    cmd = [NVCC, "-shared", GENCODE, "-o", tmp] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def clean() -> None:
    shutil.rmtree(OUT_DIR, ignore_errors=True)
    if os.path.exists(LIB):
        os.remove(LIB)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
