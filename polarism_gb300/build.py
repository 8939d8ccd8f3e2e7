"""Build libpolarism_gb300.so in-tree with nvcc for sm_103a.

``python -m polarism_gb300.build`` compiles every ``csrc/*.cu`` translation unit
in parallel and links them into ``polarism_gb300/_build/libpolarism_gb300.so``.
Objects are rebuilt only when a source or header is newer than the library.
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
BUILD = PKG / "_build"
INCLUDE = PKG.parent / "include"
LIBRARY = BUILD / "libpolarism_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE)]


def nvcc_path() -> str:
    for candidate in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build polarism_gb300")


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIBRARY.exists():
        return True
    newest = max(p.stat().st_mtime for p in [*CSRC.glob("*"), *INCLUDE.glob("*.h"), Path(__file__)])
    return newest > LIBRARY.stat().st_mtime


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link the library; return its path."""
    if not force and not _stale():
        return LIBRARY
    nvcc = nvcc_path()
    BUILD.mkdir(exist_ok=True)
    extra = os.environ.get("PG_NVCC_FLAGS", "").split()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{proc.stdout}\n{proc.stderr}")
        if verbose and proc.stderr:
            print(proc.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(sources()), os.cpu_count() or 4))) as pool:
        objects = list(pool.map(compile_one, sources()))
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objects)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"link failed:\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
