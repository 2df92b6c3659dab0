"""TEST INFRASTRUCTURE ONLY. Builds the CPU oracle (liboracle.so) and, where the vkrt sources are present, the
small reference-compiled checker in oracle/_ref/.

liboracle.so: the C++ restatement of vkrt's path-tracing shaders plus the FP64 intersector (oracle.cpp,
rgb2spec_fit.cpp), compiled with -ffp-contract=off so FP32 expressions round exactly as written.

oracle/_ref/libvkrt_ref.so: vkrt's own src/core/utility/packing.c compiled unchanged from the vkrt checkout,
linked with ref_driver.c, which calls vkrt's vendored cglm (header-only) for camera and mesh matrices. It pins the
host-side packing and matrix conventions. It is built only where the environment variable VKRT_REFERENCE names a
vkrt checkout; tests/golden/make_golden.py uses it to regenerate the golden fixtures the tests read.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_LIB = REF_DIR / "libvkrt_ref.so"
# a vkrt checkout, named by the environment; without one the reference-compiled checker is not built
VKRT_SRC = Path(os.environ["VKRT_REFERENCE"]) if os.environ.get("VKRT_REFERENCE") else None


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(map(str, cmd)) + "\n" + proc.stdout)


def _machine_changed(tag: str) -> bool:
    stamp = HERE / f".{tag}.machine"
    m = platform.machine()
    changed = not stamp.exists() or stamp.read_text().strip() != m
    stamp.write_text(m)
    return changed


def build_oracle(force: bool = False) -> Path:
    force = _machine_changed("oracle") or force
    srcs = [HERE / "oracle.cpp", HERE / "rgb2spec_fit.cpp"]
    deps = srcs + [HERE / "oracle.h", HERE / "oracle_math.h", ROOT / "include" / "vkrt_cuda.h",
                   ROOT / "include" / "vkrt_cuda_types.h"]
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in deps):
        _run(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off", f"-I{ROOT / 'include'}",
              f"-I{HERE}", *map(str, srcs), "-o", str(LIB), "-lpthread"])
    return LIB


def build_reference(force: bool = False) -> Path | None:
    if VKRT_SRC is None:
        return None
    packing = VKRT_SRC / "src/core/utility/packing.c"
    if not packing.exists():
        return None
    REF_DIR.mkdir(exist_ok=True)
    driver = HERE / "ref_driver.c"
    if force or not REF_LIB.exists() or driver.stat().st_mtime > REF_LIB.stat().st_mtime:
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
              f"-I{VKRT_SRC / 'src/shared'}", f"-I{VKRT_SRC / 'src/core/utility'}",
              f"-I{VKRT_SRC / 'external/cglm/include'}", str(packing), str(driver), "-o", str(REF_LIB), "-lm"])
    return REF_LIB


def build(force: bool = False) -> None:
    build_oracle(force)
    build_reference(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
