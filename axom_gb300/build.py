"""Builds libgsq.so (the CUDA kernels and the C ABI) for sm_103a, in-tree.

Each translation unit in ``csrc/`` is compiled to an object in ``_build/`` in
parallel, then linked into ``axom_gb300/libgsq.so``.  Device code is compiled
with ``-fmad=false`` and host code with ``-ffp-contract=off`` so that no
multiply-add is fused anywhere: the FP64 paths must round exactly as the
reference's host build does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libgsq.so"
ROOT = PKG.parent

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", f"-I{ROOT / 'include'}"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise FileNotFoundError("nvcc not found")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps_mtime() -> float:
    files = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return max(f.stat().st_mtime for f in files)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime > _deps_mtime():
        return LIB
    OBJ.mkdir(exist_ok=True)
    cc = nvcc()
    flags = NVCC_FLAGS + (extra or [])
    jobs = []
    for src in sources():
        obj = OBJ / (src.stem + ".o")
        jobs.append([cc, *flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for cmd, p in ex.map(run, jobs):
            if verbose and p.stderr:
                print(p.stderr)
            if p.returncode != 0:
                raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{p.stderr[-6000:]}")
    tmp = LIB.with_suffix(".so.tmp")
    link = [cc, *ARCH, "-shared", "-o", str(tmp)] + [str(OBJ / (s.stem + ".o")) for s in sources()]
    p = subprocess.run(link, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
