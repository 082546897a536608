"""Recipe for the reference-GPU checker (test infrastructure, not product code).

The reference runs its focal stencils as CUDA C source strings compiled at
run time (``*_KERNEL_SOURCE`` in src/vibespatial/raster/kernels/focal.py,
launched from src/vibespatial/raster/algebra.py).  This recipe

1. ``extract``: reads that module as text (``ast``; nothing of the reference
   is imported or executed) and writes each kernel source string, unchanged,
   to ``oracle/_ref/<name>.cuh`` -- a git-ignored folder, so the reference's
   sources never enter this repository's history;
2. ``compile``: builds ``oracle/_ref/libvsr_refgpu.so`` from
   ``oracle/ref_gpu_launch.cu`` (this repository's own host launchers, one
   object per kernel) with nvcc for sm_103a.  The launchers use the
   reference's launch geometry (16 x 16 blocks, its dynamic shared-memory
   sizes, algebra.py:1943-2083, 2320-2383, 2700-2760, 3239-3349).

``prepare()`` runs both steps when the sources are reachable, else only the
second (the extracted ``.cuh`` files travel with the working tree to a GPU
machine that has no copy of the reference).  Only ``tests/`` use the result.

    python oracle/make_ref_gpu.py --reference /path/to/vibespatial-raster
"""

from __future__ import annotations

import argparse
import ast
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libvsr_refgpu.so"
FOCAL = Path("src/vibespatial/raster/kernels/focal.py")
# kernel source constant -> file name; each launcher object includes one
KERNELS = {
    "CONVOLVE_NORMALIZED_KERNEL_SOURCE": "convolve_normalized",
    "SLOPE_ASPECT_KERNEL_SOURCE": "slope_aspect",
    "HILLSHADE_KERNEL_SOURCE": "hillshade",
    "FOCAL_STATS_KERNEL_SOURCE": "focal_stats",
}
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def extract(reference: Path) -> list[Path]:
    """Write the reference's kernel source strings to oracle/_ref/*.cuh."""
    src = (reference / FOCAL).read_text()
    tree = ast.parse(src)
    found = {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name):
            name = node.targets[0].id
            if name in KERNELS and isinstance(node.value, ast.Constant) and isinstance(node.value.value, str):
                found[name] = node.value.value
    missing = sorted(set(KERNELS) - set(found))
    if missing:
        raise RuntimeError(f"{reference / FOCAL}: kernel sources not found: {missing}")
    OUT.mkdir(exist_ok=True)
    paths = []
    for name, stem in KERNELS.items():
        p = OUT / f"{stem}.cuh"
        p.write_text(f"// extracted from {FOCAL} ({name}); not part of this repository\n" + found[name])
        paths.append(p)
    return paths


def compile_lib() -> Path:
    """nvcc the launchers (one object per kernel) into oracle/_ref/libvsr_refgpu.so."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    missing = [s for s in KERNELS.values() if not (OUT / f"{s}.cuh").exists()]
    if missing:
        raise RuntimeError(f"extracted kernel sources missing in {OUT}: {missing}; run extract() first")
    objs = []
    procs = []
    for stem in KERNELS.values():
        obj = OUT / f"ref_{stem}.o"
        cmd = [nvcc, GENCODE, "-O3", "-std=c++17", "-Xcompiler=-fPIC", f"-DREF_{stem.upper()}", f"-I{OUT}",
               "-c", str(HERE / "ref_gpu_launch.cu"), "-o", str(obj)]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
        objs.append(obj)
    for cmd, pr in procs:
        out, _ = pr.communicate()
        if pr.returncode:
            raise RuntimeError(f"{' '.join(cmd)} failed:\n{out}")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"linking {LIB} failed:\n{r.stdout}{r.stderr}")
    tmp.replace(LIB)
    return LIB


def prepare(reference: Path | None = None) -> Path | None:
    """Extract (when the reference is reachable) and compile; None when no sources exist."""
    if reference is not None and (reference / FOCAL).exists():
        extract(reference)
    if all((OUT / f"{s}.cuh").exists() for s in KERNELS.values()):
        return compile_lib()
    return None


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--reference", type=Path, required=True, help="root of the vibespatial-raster checkout")
    ap.add_argument("--no-compile", action="store_true", help="only extract the kernel sources")
    args = ap.parse_args(argv)
    extract(args.reference)
    if not args.no_compile:
        print(compile_lib())
    return 0


if __name__ == "__main__":
    sys.exit(main())
