"""In-tree build of librfba_srrf.so for sm_103a.

CUDA sources compile with nvcc for exactly one target (compute_103a/sm_103a),
host sources with g++; translation units compile in parallel and link with
nvcc into rfba_gb300/_lib/librfba_srrf.so (CUDA runtime linked statically, no
libcuda link dependency, so the library loads on machines without a GPU).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "librfba_srrf.so"
OBJ_DIR = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


CLI_SRC = CSRC / "cli_srrf.cpp"
CLI = OUT_DIR / "rfba-srrf"


def sources():
    """Library translation units (the command-line front end is linked separately)."""
    return sorted(CSRC.glob("*.cu")), sorted(p for p in CSRC.glob("*.cpp") if p != CLI_SRC)


def build_cli(force: bool = False) -> Path:
    """rfba-srrf: the RFBA.bat `--srrf_only 1` step on the library (rpath $ORIGIN)."""
    if CLI.exists() and not force and CLI.stat().st_mtime >= max(CLI_SRC.stat().st_mtime, LIB.stat().st_mtime):
        return CLI
    tmp = CLI.with_suffix(".tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(PKG.parent / "include"), str(CLI_SRC),
           "-o", str(tmp), "-L", str(OUT_DIR), "-lrfba_srrf", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


def _compile(src: Path, verbose_ptxas: bool) -> Path:
    obj = OBJ_DIR / (src.name + ".o")
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", str(PKG.parent / "include"), "-c", str(src), "-o", str(obj)]
        if verbose_ptxas:
            cmd[1:1] = ["-Xptxas", "-v"]
    else:
        # no floating-point contraction: host arithmetic that follows the
        # reference's (ring and window tables, the spot optimiser) gives the same
        # bits on x86 and Arm
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-I", _cuda_include(), "-I",
               str(PKG.parent / "include"), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compile when a source is newer than the library. Concurrent callers (one
    per rank) serialise on a lock file, and the later ones find it up to date."""
    import fcntl
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    with open(OUT_DIR / ".build.lock", "w") as lk:
        fcntl.flock(lk, fcntl.LOCK_EX)
        try:
            return _build_locked(force, verbose_ptxas)
        finally:
            fcntl.flock(lk, fcntl.LOCK_UN)


def _build_locked(force: bool, verbose_ptxas: bool) -> Path:
    cu, cpp = sources()
    srcs = cu + cpp
    headers = list(CSRC.glob("*.h")) + list((PKG.parent / "include").glob("*.h"))
    newest = max(p.stat().st_mtime for p in srcs + headers)
    if LIB.exists() and not force and not verbose_ptxas and LIB.stat().st_mtime >= newest:
        build_cli()
        return LIB
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli(force=True)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
