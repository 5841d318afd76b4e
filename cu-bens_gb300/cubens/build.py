"""Build the CUDA libraries in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel. All but
dropin.cu are linked into libcubens_gb300.so, which exports the C ABI of
include/cubens_gb300.h; dropin.cu becomes libcubens_dropin.so (the
prototypes.h entry points of include/cubens_gb300_dropin.h), linked against
the first with an $ORIGIN run path.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parents[1]          # cu-bens_gb300/
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libcubens_gb300.so"
DROPIN_LIB = PKG / "lib" / "libcubens_dropin.so"
DROPIN_SRC = "dropin.cu"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I", str(INCLUDE), "-I", str(CSRC)]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(p).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build cubens_gb300")
    return p


def sources() -> list[Path]:
    return sorted([*CSRC.glob("*.cu"), *CSRC.glob("*.cpp")])


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    headers = [*CSRC.glob("*.hpp"), *CSRC.glob("*.cuh"), *INCLUDE.glob("*.h")]
    objs = []
    jobs = []
    for src in sources():
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *(extra or []), "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    if jobs:
        with ThreadPoolExecutor(workers) as ex:
            for err in ex.map(run, jobs):
                if verbose and err:
                    print(err)
    main_objs = [o for o in objs if o.name != DROPIN_SRC + ".o"]
    dropin_objs = [o for o in objs if o.name == DROPIN_SRC + ".o"]
    if force or jobs or _stale(LIB, main_objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, main_objs)]
        run(cmd)
    if dropin_objs and (force or jobs or _stale(DROPIN_LIB, [*dropin_objs, LIB])):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(DROPIN_LIB), *map(str, dropin_objs), "-L", str(LIB.parent),
               "-lcubens_gb300", "-Xlinker", "-rpath,$ORIGIN"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
