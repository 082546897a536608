"""The integer float-to-double widening (csrc/df_round.h) equals the FP64 conversion.

The terrain-derivative kernel writes its float64 outputs as the sum of two
floats widened by vsr_f32_widen instead of FP64 conversions; the routine is
plain C, so this host test compiles it with gcc and compares it bit for bit
with the compiler's (double) conversion over a strided sweep of all float bit
patterns (zeros, subnormals, infinities and NaNs included).  The GPU side is
covered by the derivative parity tests.
"""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "vibespatial-raster_gb300" / "csrc"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_f32_widen_matches_conversion(tmp_path):
    exe = tmp_path / "df_round_check"
    subprocess.run(["gcc", "-O2", "-std=c99", "-I", str(CSRC), "-o", str(exe),
                    str(Path(__file__).with_name("df_round_check.c"))], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    n, accepted, bad = map(int, res.stdout.split()[-3:])
    assert bad == 0
    assert accepted > n * 0.9  # every normal float and the zeros
