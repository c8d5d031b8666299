"""Build recipe for libcapsp.so (CUDA kernels + C-ABI + host C code).

Every translation unit is compiled in parallel (nvcc for ``.cu`` with one
``-gencode arch=compute_103a,code=sm_103a``, gcc for ``.c``) and linked into
``capellinisptrsv_gb300/_build/libcapsp.so`` with the CUDA runtime linked
statically, so the library carries no dependency on torch's runtime copy.
No cmake; the whole build takes well under a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libcapsp.so"
# cuSPARSE SpSV side-by-side used by bench.py only (never by the solve path)
VENDOR_LIB = BUILD / "libcapsp_vendor.so"
# command-line driver with the reference's main.cu flow and result.csv format
CLI = BUILD / "capsp_run"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CC_FLAGS = ["-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-fopenmp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcapsp")
    return cand


def sources() -> tuple[list[Path], list[Path]]:
    cu = sorted(CSRC.glob("*.cu"))
    c = sorted((CSRC / "host").glob("*.c"))
    return cu, c


def _deps() -> list[Path]:
    cu, c = sources()
    hdrs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((CSRC / "host").glob("*.h"))
    hdrs += list((CSRC / "cli").glob("*.c"))
    return cu + c + hdrs + list((CSRC / "vendor").glob("*.cu")) + [ROOT / "include" / "capsp.h", Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists() or not CLI.exists() or (any((CSRC / "vendor").glob("*.cu")) and not VENDOR_LIB.exists()):
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({' '.join(cmd[:3])} ...):\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libcapsp.so for sm_103a if any source is newer than it."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    cu, c = sources()
    jobs = []
    objs = []
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *inc, "-c", str(src), "-o", str(obj)])
    for src in c:
        obj = BUILD / (src.stem + ".c.o")
        objs.append(obj)
        jobs.append(["gcc", *CC_FLAGS, *inc[0:2], "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    tmp = BUILD / "libcapsp.so.tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs),
          "-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    tmp_cli = BUILD / "capsp_run.tmp"
    _run(["gcc", "-std=c11", "-O2", "-Wall", "-I", str(ROOT / "include"), str(CSRC / "cli" / "capsp_run.c"),
          "-L", str(BUILD), "-lcapsp", "-Wl,-rpath,$ORIGIN", "-o", str(tmp_cli)])
    os.replace(tmp_cli, CLI)
    build_vendor(nvcc, verbose)
    return LIB


def build_vendor(nvcc: str, verbose: bool = False) -> None:
    """libcapsp_vendor.so (cuSPARSE comparison); optional: a failure only warns."""
    src = CSRC / "vendor" / "spsv_cusparse.cu"
    if not src.exists():
        return
    tmp = BUILD / "libcapsp_vendor.so.tmp"
    try:
        _run([nvcc, *ARCH, *NVCC_FLAGS, "-shared", "-cudart", "static", str(src), "-o", str(tmp), "-lcusparse"])
        os.replace(tmp, VENDOR_LIB)
        if verbose:
            print(f"built {VENDOR_LIB}", file=sys.stderr)
    except RuntimeError as e:
        print(f"warning: cuSPARSE comparison library not built: {str(e)[:200]}", file=sys.stderr)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
