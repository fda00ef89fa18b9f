"""Regenerates the committed golden fixtures of this directory.

border_tables.json
    The explicit border-copy offset tables of the reference
    (Code/Maple/src/Shaders/DDGI/BorderUpdate.glsl:25-133: 68 entries for
    the 16x16 distance probes, 36 for the 8x8 irradiance probes), read from
    the reference source as text.  Each entry is (src.x, src.y, dst.x, dst.y)
    relative to the probe cell origin.
reference_params.json
    Parameter defaults the path reads, read from the reference source as
    text: DDGIUniform / IrradianceVolume defaults (Engine/DDGI/DDGIRenderer.h),
    the octahedral sides, and the march step cap (Shaders/SDF/SDFCommon.glsl).

Run from the repository root with the path of a reference checkout:
    python tests/golden/make_golden.py /path/to/reference
(or with the checkout in $LUXGI_REFERENCE).
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

import os

_ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LUXGI_REFERENCE")
if not _ref:
    sys.exit("usage: make_golden.py /path/to/reference (or set LUXGI_REFERENCE)")
REF = Path(_ref)
OUT = Path(__file__).resolve().parent
SH = REF / "Code/Maple/src/Shaders"
ENG = REF / "Code/Maple/src/Engine"


def border_tables() -> dict:
    text = (SH / "DDGI/BorderUpdate.glsl").read_text()
    tables = {}
    for m in re.finditer(r"const ivec4 Offsets\[(\d+)\]\s*=\s*ivec4\[\]\((.*?)\);", text, re.S):
        n = int(m.group(1))
        entries = [list(map(int, e)) for e in re.findall(r"ivec4\(\s*(-?\d+),\s*(-?\d+),\s*(-?\d+),\s*(-?\d+)\)", m.group(2))]
        assert len(entries) == n, (n, len(entries))
        side = 16 if n == 68 else 8
        tables[str(side)] = entries
    assert set(tables) == {"8", "16"}
    return {"source": "Code/Maple/src/Shaders/DDGI/BorderUpdate.glsl:25-133",
            "layout": "src.x, src.y, dst.x, dst.y relative to cell origin (BorderUpdate.glsl:136-146)",
            "tables": tables}


def reference_params() -> dict:
    h = (ENG / "DDGI/DDGIRenderer.h").read_text()
    def num(pat, text=h):
        m = re.search(pat, text)
        assert m, pat
        return float(m.group(1).rstrip("f"))
    uni = h[h.index("struct DDGIUniform"):h.index("struct IrradianceVolume")]
    vol = h[h.index("struct IrradianceVolume"):]
    sdf = (SH / "SDF/SDFCommon.glsl").read_text()
    return {
        "source": ["Code/Maple/src/Engine/DDGI/DDGIRenderer.h:17-60", "Code/Maple/src/Shaders/SDF/SDFCommon.glsl:8,143"],
        "irradiance_oct_size": int(num(r"IrradianceOctSize\s*=\s*(\d+)")),
        "depth_oct_size": int(num(r"DepthOctSize\s*=\s*(\d+)")),
        "uniform": {
            "max_distance": num(r"maxDistance\s*=\s*([\d.]+f?)", uni),
            "sharpness": num(r"depthSharpness\s*=\s*([\d.]+f?)", uni),
            "hysteresis": num(r"hysteresis\s*=\s*([\d.]+f?)", uni),
            "normal_bias": num(r"normalBias\s*=\s*([\d.]+f?)", uni),
            "ddgi_gamma": num(r"ddgiGamma\s*=\s*([\d.]+f?)", uni),
            "rays_per_probe": int(num(r"raysPerProbe\s*=\s*(\d+)", uni)),
        },
        "volume": {
            "probe_distance": num(r"probeDistance\s*=\s*([\d.]+f?)", vol),
            "rays_per_probe": int(num(r"raysPerProbe\s*=\s*(\d+)", vol)),
            "hysteresis": num(r"hysteresis\s*=\s*([\d.]+f?)", vol),
            "intensity": num(r"intensity\s*=\s*([\d.]+f?)", vol),
            "normal_bias": num(r"normalBias\s*=\s*([\d.]+f?)", vol),
            "sharpness": num(r"depthSharpness\s*=\s*([\d.]+f?)", vol),
            "ddgi_gamma": num(r"ddgiGamma\s*=\s*([\d.]+f?)", vol),
        },
        "global_sdf_world_size": num(r"GLOBAL_SDF_WORLD_SIZE\s+([\d.]+f?)", sdf),
        "max_march_steps": int(num(r"step\s*<\s*(\d+)\s*&&", sdf)),
    }


if __name__ == "__main__":
    (OUT / "border_tables.json").write_text(json.dumps(border_tables(), separators=(",", ":")) + "\n")
    (OUT / "reference_params.json").write_text(json.dumps(reference_params(), indent=1) + "\n")
    print("wrote", OUT / "border_tables.json", OUT / "reference_params.json")
