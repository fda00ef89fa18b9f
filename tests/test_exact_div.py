"""The march's exact quotient (xdiv, luxgi_common.cuh) against IEEE division.

The march divides by loop-fixed divisors every step: the cascade's extent
2 cw, the cascade count and the voxel size (SDFCommon.glsl:64-71 and the
thickness test of tracyGlobalSDF).  Its quotients must round exactly like
the CPU restatement's divisions for the march to stay bit-exact, so the
kernel forms them from y = RN(1 / d) with two fused corrections.  The
sequence is restated in `exact_div_check.c` and checked there over every
significand of the dividend (both signs, several binades, signed zeros)
for the divisors below: the engine's default cascade extents
(GlobalDistanceField.cpp:599-661: 40, 100, 200, 400 m at 256^3), the test
and bench scenes' extents, and significands at the edges (all ones, one
past one)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent

DIVISORS = [
    # engine defaults: 2 x cascade distance and its voxel size at 256^3
    "80", "200", "400", "800", "0.3125", "0.78125", "1.5625", "3.125",
    # scenes of the tests and the bench: 10 m and 60 m rooms, the inner cascade of a
    # 2-cascade 24 m room at 32^3, a 3-cascade volume's cascade count
    "10", "60", "0.234375", "9.6", "0.3", "3",
    # edge significands and arbitrary ones
    "1.99999988079071044921875", "1.00000011920928955078125", "1.7320508", "1.4142135", "2.7182817",
    "0.1", "0.7", "12345.678",
]


def test_exact_quotient_matches_ieee_division(tmp_path):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "exact_div_check"
    subprocess.run([cc, "-O2", "-fopenmp", "-ffp-contract=off", str(HERE / "exact_div_check.c"), "-o", str(exe),
                    "-lm"], check=True)
    r = subprocess.run([str(exe), *DIVISORS], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
