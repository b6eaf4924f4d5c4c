"""Build recipe for the CPU oracle library (test infrastructure only).

Compiles ``oracle/oracle.cpp`` with g++ and OpenMP into ``oracle/liboracle.so``.
FMA contraction is disabled so the FP64 arithmetic follows the reference's
Numba kernels operation by operation on both x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "oracle.cpp"
LIBRARY = HERE / "liboracle.so"

FLAGS = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the oracle if the shared library is missing or older than its source."""
    if not force and LIBRARY.exists() and LIBRARY.stat().st_mtime >= SOURCE.stat().st_mtime:
        return LIBRARY
    tmp = LIBRARY.with_suffix(f".so.tmp{os.getpid()}")
    cmd = ["g++", *FLAGS, str(SOURCE), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
