"""Host-side contracts that drift silently if one side changes (CPU only).

* the autotuner's configuration table mirrors the compiled Horn table, and the
  library reports the same count;
* the tuning cache round-trips through its JSON file and keys by size class;
* the ctypes mirror of ``vsr_batch_tile`` has the C header's layout (checked by
  compiling the header with gcc and printing ``offsetof``).
"""

from __future__ import annotations

import ctypes
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from vsr_gb300 import _build, _lib

    _build.build()
    return _lib.load()


def test_horn_config_table_mirrors_the_library(lib):
    from vsr_gb300 import _lib, autotune

    src = (ROOT / "vibespatial-raster_gb300" / "csrc" / "horn.cu").read_text()
    body = re.search(r"kHornConfigs\[\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    table = [tuple(int(v) for v in t.split(",")) for t in re.findall(r"\{([^{}]*)\}", body)]
    assert table == [tuple(c) for c in autotune.HORN_CONFIGS]
    assert lib.vsr_tuning_count(_lib.VSR_OP_HORN) == len(table)
    # out-of-range choices are refused on the host
    assert lib.vsr_tuning_set(_lib.VSR_OP_HORN, len(table)) == _lib.VSR_ERR_INVALID_ARG
    assert lib.vsr_tuning_set(99, 0) == _lib.VSR_ERR_INVALID_ARG


def test_tuning_cache_round_trip(tmp_path, monkeypatch):
    from vsr_gb300 import autotune

    monkeypatch.setenv("VSR_GB300_CACHE", str(tmp_path))
    assert autotune._load_cache() == {}
    autotune._store_cache({"horn|16384x16384|float32|sm152": {"config": 1, "ms": {"0": 0.7}}})
    assert autotune._load_cache()["horn|16384x16384|float32|sm152"]["config"] == 1
    assert (tmp_path / "tuning.json").exists()
    # size classes: the next power of two of each side
    assert autotune._size_class(16384, 16384) == "16384x16384"
    assert autotune._size_class(10980, 300) == "16384x512"
    assert autotune._size_class(1, 1) == "1x1"


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_batch_tile_layout_matches_the_header(tmp_path):
    from vsr_gb300.batch import BatchTile

    fields = [f for f, _ in BatchTile._fields_]
    prog = tmp_path / "layout.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "vsr.h"\nint main(void) {\n'
        '  printf("%zu\\n", sizeof(vsr_batch_tile));\n'
        + "".join(f'  printf("%zu\\n", offsetof(vsr_batch_tile, {f}));\n' for f in fields)
        + "  return 0;\n}\n"
    )
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(prog), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert out[0] == ctypes.sizeof(BatchTile)
    assert out[1:] == [getattr(BatchTile, f).offset for f in fields]
