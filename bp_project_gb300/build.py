"""Build libsarbp.so (the sm_103a CUDA kernels + C ABI) in-tree.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc for
``sm_103a`` only, then linked into ``bp_project_gb300/libsarbp.so`` with the
CUDA runtime linked statically.  No CMake, no torch extension machinery: the
library exports the plain C ABI declared in ``include/sarbp.h``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
REPO = PACKAGE.parent
CSRC = PACKAGE / "csrc"
INCLUDE = REPO / "include"
BUILD = PACKAGE / "_build"
LIBRARY = PACKAGE / "libsarbp.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(INCLUDE), "-I", str(CSRC)]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libsarbp")
    return path


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIBRARY.exists():
        return True
    built = LIBRARY.stat().st_mtime
    deps = [*sources(), *CSRC.glob("*.cuh"), *INCLUDE.glob("*.h"), Path(__file__)]
    return any(p.stat().st_mtime > built for p in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False, bulk_windows: bool = False) -> Path:
    """Compile and link libsarbp.so if any source is newer than the library.

    ``bulk_windows`` builds the measured alternative in which the direct kernels' range windows
    arrive in shared memory by cp.async.bulk copies (SARBP_BULK_WINDOWS); it is 2% slower than the
    default on the 4096-pulse lattice and is not the default.  Rebuild with force=True to switch."""
    if not force and not _stale():
        return LIBRARY
    BUILD.mkdir(exist_ok=True)
    compiler = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    if bulk_windows:
        extra += ["-DSARBP_BULK_WINDOWS=1"]

    def compile_one(src: Path):
        obj = BUILD / (src.stem + ".o")
        cmd = [compiler, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        if ptxas_info or verbose:
            sys.stderr.write(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as pool:
        objects = list(pool.map(compile_one, sources()))
    tmp = LIBRARY.with_name(f"libsarbp.so.tmp{os.getpid()}")
    cmd = [compiler, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objects)]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv,
                bulk_windows="--bulk-windows" in sys.argv))
