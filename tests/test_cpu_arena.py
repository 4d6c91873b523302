"""The HBM arena's host bookkeeping under concurrent use (no device memory
is touched): blocks never overlap, stay aligned inside the slab, can be freed
by another thread, and the used count returns to zero.  An allocation that
does not fit runs the reclaim hook (deferred releases) before it fails, and the
peak covers the largest use seen.  Regions return to the arena with their
last reference, whichever thread drops it."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


@pytest.fixture(scope="module")
def arena_check(tmp_path_factory):
    if not shutil.which("g++") or not os.path.exists(os.path.join(CUDA, "include", "cuda_runtime.h")):
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path_factory.mktemp("arena") / "arena_check")
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I" + os.path.join(CUDA, "include"),
           os.path.join(ROOT, "tests", "arena_check.cpp"),
           os.path.join(ROOT, "vedas_gb300", "csrc", "vg_ctx.cpp"),
           "-L" + os.path.join(CUDA, "lib64"), "-lcudart_static", "-ldl", "-lrt", "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("threads,ops", [(1, 200_000), (8, 60_000), (16, 30_000)])
def test_arena_concurrent_bookkeeping(arena_check, threads, ops):
    r = subprocess.run([arena_check, str(threads), str(ops)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "overlaps_or_out_of_range=0" in r.stdout
    assert "reclaim_ok=1 peak_ok=1 region_ok=1" in r.stdout
