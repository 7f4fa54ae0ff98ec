"""In-tree build of the native library (libgst.so) for sm_103a.

Compiles the CUDA/C++ sources under csrc/ with nvcc (one -gencode, sm_103a)
and g++, in parallel, and links them into gpu4gst_code_gb300/_lib/libgst.so
with the CUDA runtime linked statically. Rebuilds whenever the content of a
source, a header, the flags, the host architecture or the toolkit differs
from what the library was built from (a SHA-256 stamp written beside it),
so a library copied from another machine or built from other sources is
never reused. No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = ROOT / "_build" / "gst"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libgst.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC"]

CU_SOURCES = ["dpbf_kernels.cu", "learn_kernels.cu", "engine.cu", "noalloc.cu"]
CXX_SOURCES = ["gen.cpp", "dataset.cpp"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgst")
    return cand


def toolkit_available() -> bool:
    return bool(shutil.which("nvcc")) or Path("/usr/local/cuda/bin/nvcc").exists()


def _inputs() -> list[Path]:
    files = [CSRC / s for s in CU_SOURCES + CXX_SOURCES]
    files += sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.hpp")) + sorted(INCLUDE.glob("*.h"))
    files.append(Path(__file__))
    return files


STAMP = LIB.with_suffix(".so.sha256")


def _digest(inputs: list[Path]) -> str:
    """SHA-256 over every input's name and bytes, the flags, the host
    architecture and the nvcc binary's path and size."""
    h = hashlib.sha256()
    h.update(" ".join(ARCH + NVCC_FLAGS + CXX_FLAGS + CU_SOURCES + CXX_SOURCES).encode())
    h.update(platform.machine().encode())
    try:
        nv = Path(nvcc())
        h.update(f"{nv}:{nv.stat().st_size}".encode())
    except (RuntimeError, OSError):
        pass
    for p in inputs:
        h.update(p.name.encode())
        h.update(p.read_bytes() if p.exists() else b"<missing>")
    return h.hexdigest()


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists() or not STAMP.exists():
        return True
    return STAMP.read_text().strip() != _digest(inputs)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Builds libgst.so if needed and returns its path."""
    inputs = _inputs()
    if not force and not _stale(LIB, inputs):
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    nv = nvcc()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        jobs.append([nv, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        cxx = shutil.which("g++") or "g++"
        jobs.append([cxx, *CXX_FLAGS, "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nv, *ARCH, "-shared", "-cudart", "static", *map(str, objs), "-o", str(tmp)])
    os.replace(tmp, LIB)
    STAMP.write_text(_digest(inputs) + "\n")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build_library(force=True, verbose=True)
