"""Builds the native libraries in-tree.

libluxgi_ddgi.so  the CUDA kernels and the C ABI (nvcc, sm_103a only)
libluxgi_scene.so the synthetic scene generator (g++, OpenMP)

Both land in luxgi_gb300/lib/.  Rebuilds only what is older than its sources.
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
INCLUDE = ROOT / "include"
LIB = PKG / "lib"
OBJ = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# translation units whose FP32 arithmetic must match the CPU restatement bit
# for bit are built without FMA contraction
NO_FMAD = {"trace.cu", "setup.cu", "surface.cu", "sdfbuild.cu"}
# shading is compared with the restatement by tolerance: approximate
# division and square root, denormals flushed to zero (the special-function
# results need no denormal fix-ups; no shading quantity is near 1e-38)
FAST_DIV = {"shade.cu"}
# host code built without FMA contraction, so that its results (the seeded
# frame rotations) are the same on x86 and aarch64 hosts
HOST_NO_CONTRACT = {"capi.cu"}
CUDA_SOURCES = ["trace.cu", "shade.cu", "blend.cu", "blend_tc.cu", "setup.cu", "surface.cu", "sdfbuild.cu", "capi.cu",
                "batch.cu", "server.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def build_cuda(verbose: bool = False) -> Path:
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    out = LIB / "libluxgi_ddgi.so"
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE),
                   "-I", str(CSRC), "-c", str(s), "-o", str(o)]
            if src in NO_FMAD:
                # device code without FMA contraction, and the host code too
                # (gcc contracts by default on aarch64)
                cmd[1:1] = ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]
            if src in HOST_NO_CONTRACT:
                cmd[1:1] = ["-Xcompiler", "-ffp-contract=off"]
            if src in FAST_DIV:
                cmd[1:1] = ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if _stale(out, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcuda"])
    return out


def build_scene() -> Path:
    LIB.mkdir(exist_ok=True)
    out = LIB / "libluxgi_scene.so"
    src = CSRC / "scene.cpp"
    if _stale(out, [src] + _headers()):
        _run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-I", str(INCLUDE),
              str(src), "-o", str(out)])
    return out


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_cuda, verbose)
        b = ex.submit(build_scene)
        a.result()
        b.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIB)
