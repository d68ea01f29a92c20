"""Injected allocation failure on the host (no GPU needed).

The context's scratch buffers (rfba_gb300/csrc/devbuf.h) honour
RFBA_TEST_ALLOC_FAIL=k: the k-th allocation after the variable takes that value
fails as an out-of-memory would, once. This drives the real header from a small
C++ program: the injected allocation reports RFBA_ERR_NOMEM (-3) with the
buffer's name, and the allocations around it are untouched (on a machine
without a GPU they fail with RFBA_ERR_CUDA (-4), on one with a GPU they
succeed). tests/test_zz_alloc_failure_gpu.py checks the same hook through the
C-ABI on a GPU, including that the next call on the same context succeeds.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "native" / "alloc_hook_check.cpp"


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("CUDA toolkit not present")
    cuda = Path(nvcc).resolve().parent.parent
    out = tmp_path_factory.mktemp("alloc") / "alloc_hook_check"
    cmd = ["g++", "-O1", "-std=c++17", "-I", str(cuda / "include"), str(SRC), "-o", str(out),
           "-L", str(cuda / "lib64"), "-lcudart_static", "-lpthread", "-ldl", "-lrt"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def _run(prog, k, n):
    r = subprocess.run([str(prog), str(k), str(n)], capture_output=True, text=True, timeout=120, check=True)
    rows = []
    for line in r.stdout.splitlines():
        status, _, msg = line.partition(" ")
        rows.append((int(status), msg))
    return rows


def test_kth_allocation_fails_once_with_its_name(prog):
    rows = _run(prog, 3, 5)
    assert len(rows) == 5
    status, msg = rows[2]
    assert status == -3, rows
    assert msg.startswith("buffer 3:") and "RFBA_TEST_ALLOC_FAIL" in msg
    for i in (0, 1, 3, 4):
        assert rows[i][0] in (0, -4), rows  # untouched: success with a GPU, CUDA error without
        assert "RFBA_TEST_ALLOC_FAIL" not in rows[i][1]


def test_first_allocation_and_unset_variable(prog):
    rows = _run(prog, 1, 2)
    assert rows[0][0] == -3 and rows[1][0] in (0, -4)
    rows = _run(prog, 0, 2)  # 0 (or empty) injects nothing
    assert all(s in (0, -4) for s, _ in rows)
