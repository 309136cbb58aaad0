"""In-tree build of libhx.so (sm_103a) and of the CPU oracle library.

Usage: python -m hashinator_gb300.build  (or hashinator_gb300.build.build_all())

The CUDA translation units are compiled in parallel with one -gencode
(compute_103a -> sm_103a) and linked into hashinator_gb300/libhx.so. The
oracle (oracle/hx_oracle.c) is compiled with the host C compiler into
oracle/liboracle.so; it is test infrastructure only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libhx.so"

CUDA_SOURCES = ["hx_map.cu", "hx_scan.cu", "hx_batch.cu", "hx_serve.cu", "hx_noalloc.cu"]
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhx.so")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_lib(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = (sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").glob("*.h"))
               + sorted((ROOT / "include").glob("*.cuh")))
    srcs = [CSRC / s for s in CUDA_SOURCES if (CSRC / s).exists()]
    objs = []
    procs = []
    for src in srcs:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {s}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    if force or _stale(LIB, objs):
        cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", str(LIB), *map(str, objs), "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


def build_oracle(verbose: bool = False, force: bool = False) -> Path:
    """Compile the C oracle (test infrastructure) into oracle/liboracle.so."""
    src = ROOT / "oracle" / "hx_oracle.c"
    out = ROOT / "oracle" / "liboracle.so"
    if force or _stale(out, [src, ROOT / "oracle" / "hx_oracle.h"]):
        cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
        cmd = [cc, "-O2", "-std=c11", "-shared", "-fPIC", "-o", str(out), str(src)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return out


def build_all(verbose: bool = False, force: bool = False) -> None:
    build_lib(verbose=verbose, force=force)
    build_oracle(verbose=verbose, force=force)


if __name__ == "__main__":
    build_all(verbose=True, force="--force" in sys.argv)
