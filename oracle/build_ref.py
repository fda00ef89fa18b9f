"""ORACLE -- test infrastructure only.

Builds oracle/_ref/libref.so: the reference's own GLSL function libraries
compiled as C++ on the host, as a second CPU reference for the restatement
in oracle/oracle.cpp.

Compiled from the sources where they lie under the reference checkout:
    Code/Maple/src/Shaders/DDGI/DDGICommon.glsl
    Code/Maple/src/Shaders/Common/Math.glsl
    Code/Maple/src/Shaders/Raytraced/Random.glsl
    Code/Maple/src/Shaders/SDF/SDFCommon.glsl (+ ObjectRasterizeData.glsl,
        GlobalSDFData.glsl, GlobalSDFHit.glsl, GlobalSDFTrace.glsl)
    Code/Maple/src/Shaders/SDF/AtlasCommon.glsl
    Code/Maple/src/Shaders/Raytraced/BRDF.glsl (+ Raytraced/Common.glsl)
    Code/Maple/src/Shaders/Common/Light.glsl
The only change made to the text is mechanical: GLSL `out T x` / `inout T x`
parameters become C++ references `T& x` (everything else -- swizzles,
built-ins, samplers, `in` -- is supplied by oracle/glsl_compat.h).  The
rewritten text goes to a temporary directory that is deleted after the
compile; nothing of the reference source is kept in the repository tree.
The shader entry points (GISDFRays.comp main, ProbeUpdate.glsl main,
GlobalSDFMipmap.comp main, SDFCulling.comp main, SDFDeferredLight.frag
main and fetchLight, CopyEmissive.frag main, SDFAtlasIndirectLight.frag
main) use Vulkan resource
declarations that do not compile as C++, so oracle/ref_harness.cpp restates
those bodies around the compiled library functions.

Usage: python oracle/build_ref.py /path/to/reference
(or with the checkout in $LUXGI_REFERENCE)
"""
from __future__ import annotations

import itertools
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref.so"
SHADERS = ["DDGI/DDGICommon.glsl", "Common/Math.glsl", "Raytraced/Random.glsl", "SDF/SDFCommon.glsl",
           "SDF/ObjectRasterizeData.glsl", "SDF/GlobalSDFData.glsl", "SDF/GlobalSDFHit.glsl",
           "SDF/GlobalSDFTrace.glsl", "SDF/AtlasCommon.glsl", "Raytraced/Common.glsl", "Raytraced/BRDF.glsl",
           "Common/Light.glsl"]


CHECKOUT = OUT / "checkout.txt"        # the checkout the library was built from


def reference_root(arg: str | None = None) -> Path | None:
    """The reference checkout: the argument, else $LUXGI_REFERENCE, else the
    checkout the last build recorded, else None (then only a previously
    built library, if any, is used)."""
    import os

    p = arg or os.environ.get("LUXGI_REFERENCE")
    if not p and CHECKOUT.exists():
        p = CHECKOUT.read_text().strip()
    return Path(p) if p else None


def swizzles(n: int) -> str:
    """Union members for every 2-, 3- and 4-component swizzle of an n-vector."""
    xyzw, rgba = "xyzw", "rgba"
    lines = []
    for length in (2, 3, 4):
        for combo in itertools.product(range(n), repeat=length):
            idx = ", ".join(map(str, combo))
            lines.append(f"SWZ({idx}) {''.join(xyzw[i] for i in combo)};")
            lines.append(f"SWZ({idx}) {''.join(rgba[i] for i in combo)};")
    return "\n".join(lines) + "\n"


_PARAM = re.compile(r"\b(out|inout)\s+([A-Za-z_]\w*)\s+([A-Za-z_]\w*)")
# GLSL brings a variable into scope after its initializer, C++ before it:
# `ivec3 f = f(...)` must call the global function f
_SELF_INIT = re.compile(r"\b([A-Za-z_]\w*)\s+([A-Za-z_]\w*)\s*=\s*\2\s*\(")


def rewrite(text: str) -> str:
    text = _PARAM.sub(lambda m: f"{m.group(2)}& {m.group(3)}", text)
    return _SELF_INIT.sub(lambda m: f"{m.group(1)} {m.group(2)} = ::{m.group(2)}(", text)


def build(ref: Path | None = None, force: bool = False) -> Path | None:
    ref = reference_root(None if ref is None else str(ref))
    shaders = None if ref is None else ref / "Code/Maple/src/Shaders"
    if shaders is None or not shaders.is_dir():
        return LIB if LIB.exists() else None
    deps = [shaders / s for s in SHADERS] + [HERE / "glsl_compat.h", HERE / "packed_color.h", HERE / "ref_harness.cpp",
                                             HERE.parent / "include" / "luxgi_ddgi.h", Path(__file__)]
    if LIB.exists() and not force and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        CHECKOUT.write_text(str(ref.resolve()) + "\n")
        return LIB
    OUT.mkdir(exist_ok=True)
    tmp = Path(tempfile.mkdtemp(prefix="luxgi_ref_"))
    try:
        for n in (2, 3, 4):
            (tmp / f"glsl_swizzles_{n}.inc").write_text(swizzles(n))
        for s in SHADERS:
            dst = tmp / "Shaders" / s
            dst.parent.mkdir(parents=True, exist_ok=True)
            dst.write_text(rewrite((shaders / s).read_text()))
        cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-fsingle-precision-constant",
               "-ffp-contract=off", "-w", "-I", str(tmp), "-I", str(tmp / "Shaders"), "-I", str(HERE),
               "-I", str(HERE.parent / "include"), str(HERE / "ref_harness.cpp"), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + r.stderr[-6000:])
        CHECKOUT.write_text(str(ref.resolve()) + "\n")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return LIB


if __name__ == "__main__":
    p = build(Path(sys.argv[1]) if len(sys.argv) > 1 else None, force=True)
    print("built", p)
