"""Build recipe for libvsr.so (sm_103a), compiled in-tree with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel to an object file
under ``_native/_build/`` and the objects are linked into
``_native/libvsr.so``.  Only one ``-gencode`` (compute_103a -> sm_103a) is
emitted: the library targets GB300 alone.  Re-running is incremental (a unit
is rebuilt when it or any header is newer than its object).
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
SRC_DIR = PKG_DIR.parent / "csrc"
INCLUDE_DIR = PKG_DIR.parents[1] / "include"
NATIVE_DIR = PKG_DIR / "_native"
BUILD_DIR = NATIVE_DIR / "_build"
LIB_PATH = NATIVE_DIR / "libvsr.so"

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libvsr")
    return cand


def _flags(extra: list[str] | None = None) -> list[str]:
    f = [
        GENCODE,
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler=-fPIC,-O3,-fvisibility=hidden",
        "--expt-relaxed-constexpr",
        f"-I{INCLUDE_DIR}",
        f"-I{SRC_DIR}",
    ]
    if extra:
        f += extra
    return f


def _stale(obj: Path, src: Path, headers: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in headers)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compile and link libvsr.so; returns its path."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(SRC_DIR.glob("*.cu"))
    headers = sorted(SRC_DIR.glob("*.cuh")) + sorted(SRC_DIR.glob("*.h")) + sorted(INCLUDE_DIR.glob("*.h"))
    extra = ["-Xptxas=-v"] if ptxas_verbose else []
    jobs = []
    for src in sources:
        obj = BUILD_DIR / (src.stem + ".o")
        if force or ptxas_verbose or _stale(obj, src, headers):
            jobs.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc(), *_flags(extra), "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, cmd, r

    failed = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for src, cmd, r in ex.map(compile_one, jobs):
            if verbose or ptxas_verbose or r.returncode:
                sys.stderr.write(f"[vsr build] {' '.join(cmd)}\n{r.stdout}{r.stderr}")
            if r.returncode:
                failed.append(src.name)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    objs = [BUILD_DIR / (s.stem + ".o") for s in sources]
    if force or jobs or not LIB_PATH.exists() or any(o.stat().st_mtime > LIB_PATH.stat().st_mtime for o in objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [nvcc(), GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-ldl", "-lpthread", "-lrt",
               "-Xlinker", "--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(f"[vsr build] {' '.join(cmd)}\n{r.stdout}{r.stderr}")
        if r.returncode:
            raise RuntimeError("linking libvsr.so failed")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB_PATH)
