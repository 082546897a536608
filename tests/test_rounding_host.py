"""Host checks of the rounding helpers the kernels share with C (plain C headers).

* csrc/df_round.h: the terrain-derivative kernel writes its float64 outputs
  as the sum of two floats widened by vsr_f32_widen instead of FP64
  conversions; compared bit for bit with the compiler's (double) conversion
  over a strided sweep of all float bit patterns (zeros, subnormals,
  infinities and NaNs included).
* csrc/std_round.h: the 8/16-bit focal std with a float32 output is
  sqrt(N)/n rounded to float32 by vsr_std_f32 (exact integer midpoint
  tests, no FP64); compared with a long-double reference over random and
  edge-case (N, n), perfect squares included.

* csrc/terrain_exact.h: TRI and TPI of float32 windows whose values share a
  narrow binade range as exact integers, written as float64 bits; compared
  bit for bit with the reference's float64 formulas on random DEM-like,
  negative and tiny windows.

The GPU side is covered by the derivative and focal-statistics parity tests.
"""

import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "vibespatial-raster_gb300" / "csrc"

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")


def _run(tmp_path, source: str, *args: str) -> list[int]:
    exe = tmp_path / Path(source).stem
    subprocess.run(["gcc", "-O2", "-std=gnu11", "-I", str(CSRC), "-o", str(exe),
                    str(Path(__file__).with_name(source)), "-lm"], check=True)
    res = subprocess.run([str(exe), *args], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    return [int(v) for v in res.stdout.split()[-3:]]


def test_f32_widen_matches_conversion(tmp_path):
    n, accepted, bad = _run(tmp_path, "df_round_check.c")
    assert bad == 0
    assert accepted > n * 0.9  # every normal float and the zeros


def test_std_f32_is_correctly_rounded(tmp_path):
    *_, n, bad = _run(tmp_path, "std_round_check.c", "2000000")
    assert n == 2000000 and bad == 0


def test_exact_tri_tpi_match_float64(tmp_path):
    n, accepted, bad = _run(tmp_path, "terrain_exact_check.c", "2000000")
    assert bad == 0
    assert accepted > n // 2  # DEM-like windows take the integer path
