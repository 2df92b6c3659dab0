"""Build of the native library libvkrt_gb300.so (CUDA kernels for sm_103a + the C host layer).

nvcc compiles every translation unit in parallel, then links one shared object in-tree next to this file. No cmake,
no torch extension machinery: the product is a plain C-ABI library.
"""
from __future__ import annotations

import concurrent.futures as futures
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libvkrt_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["bvh_build.cu", "render.cu", "wavefront.cu", "adjoint.cu", "nrc.cu", "overlay.cu", "capi.cu",
              "noalloc.cu"]
C_SOURCES = ["host/scene_host.c"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvkrt_gb300.so")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile and link libvkrt_gb300.so if any source is newer than it. Returns the library path."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    # objects built on another machine architecture are never reused
    stamp = BUILD / "machine.txt"
    machine = platform.machine()
    if not stamp.exists() or stamp.read_text().strip() != machine:
        force = True
        stamp.write_text(machine)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    common = ["-O3", "-std=c++17", "-lineinfo", f"-I{INCLUDE}", f"-I{CSRC}", "-Xcompiler", "-fPIC"]
    jobs = []
    objects = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (Path(src).stem + ".o")
        objects.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, *common, "-c", str(s), "-o", str(o)])
    for src in C_SOURCES:
        s = CSRC / src
        o = BUILD / (Path(src).stem + ".o")
        objects.append(o)
        if force or _stale(o, [s] + headers):
            # host C is compiled without floating-point contraction so mesh matrices round as written
            jobs.append(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", f"-I{INCLUDE}", "-c", str(s),
                         "-o", str(o)])
    if jobs:
        with futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    if force or jobs or _stale(LIB, objects):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objects), "-lm"])
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
