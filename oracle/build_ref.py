"""Recipe: compile LLNL/axom's own SEQ spatial-query path into ``oracle/_ref/``.

Test infrastructure only.  This builds the *reference implementation* (axom
v0.11.0, ``spin::BVH<3,SEQ_EXEC,double>`` and ``quest::SignedDistance<3,
SEQ_EXEC>``) directly from the mounted reference sources, plus the small
``extern "C"`` shim in ``oracle/ref_shim.cpp``, into
``oracle/_ref/libaxom_ref.so``.  Nothing from the reference tree is copied
into the repository: the generated configuration headers (the files axom's
CMake would write) go to ``oracle/_ref/gen`` and the objects to
``oracle/_ref/obj``; both are git-ignored.

The reference's own build system (CMake + BLT) is not used: BLT is an empty
submodule here, and RAJA/Umpire/MPI are absent, so only ``SEQ_EXEC`` exists.
Flags follow the reference's defaults for a host build with FMA contraction
off (``-ffp-contract=off``), so the arithmetic is plain IEEE double.

Usage:  python oracle/build_ref.py [--reference /path/to/axom] [-j N]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# Where the reference tree is mounted: AXOM_REFERENCE_DIR or --reference, else
# the mount point of the container this recipe runs in (this file is the only
# one that names it; the GPU host has no reference tree and never builds it).
DEFAULT_REFERENCE = Path(os.environ.get("AXOM_REFERENCE_DIR") or "/root/reference")
OUT = HERE / "_ref"
GEN = OUT / "gen"
OBJ = OUT / "obj"
LIB = OUT / "libaxom_ref.so"

# Components whose unified headers (axom/<comp>.hpp) the sources include.
UNIFIED = ("core", "slic", "mint", "primal")

# Translation units of the SEQ path (core, slic, the mint mesh model that
# SignedDistance reads, and quest/SignedDistance.cpp).
SOURCES = [
    "axom/core/utilities/Annotations.cpp",
    "axom/core/utilities/FileUtilities.cpp",
    "axom/core/utilities/StringUtilities.cpp",
    "axom/core/utilities/System.cpp",
    "axom/core/utilities/Utilities.cpp",
    "axom/core/Types.cpp",
    "axom/core/Path.cpp",
    "axom/slic/core/Logger.cpp",
    "axom/slic/core/LogStream.cpp",
    "axom/slic/interface/slic.cpp",
    "axom/slic/internal/stacktrace.cpp",
    "axom/slic/streams/GenericOutputStream.cpp",
    "axom/mint/mesh/internal/MeshHelpers.cpp",
    "axom/mint/mesh/CurvilinearMesh.cpp",
    "axom/mint/mesh/FieldData.cpp",
    "axom/mint/mesh/Mesh.cpp",
    "axom/mint/mesh/MeshCoordinates.cpp",
    "axom/mint/mesh/ParticleMesh.cpp",
    "axom/mint/mesh/RectilinearMesh.cpp",
    "axom/mint/mesh/StructuredMesh.cpp",
    "axom/mint/mesh/UniformMesh.cpp",
    "axom/mint/utils/vtk_utils.cpp",
    "axom/mint/fem/FiniteElement.cpp",
    "axom/quest/SignedDistance.cpp",
    "axom/quest/readers/STLReader.cpp",
]

ENABLED = {
    "AXOM_USE_CLI11", "AXOM_USE_FMT", "AXOM_USE_SPARSEHASH", "AXOM_USE_MINT",
    "AXOM_USE_PRIMAL", "AXOM_USE_QUEST", "AXOM_USE_SLIC", "AXOM_USE_SLAM",
    "AXOM_USE_SPIN", "AXOM_DEPRECATED_TYPES_N", "SPARSEHASH_HASHFUN_HEADER",
    "SPARSEHASH_HASHFUN_NAMESPACE",
}
VALUES = {
    "AXOM_VERSION_MAJOR": "0", "AXOM_VERSION_MINOR": "11", "AXOM_VERSION_PATCH": "0",
    "AXOM_VERSION_FULL": "v0.11.0", "AXOM_SRC_DIR_NATIVE": "", "AXOM_BIN_DIR_NATIVE": "",
    "BLT_CXX_STD": "c++17", "AXOM_DEPRECATED_TYPES_N": "2",
    "SPARSEHASH_HASHFUN_HEADER": "<functional>", "SPARSEHASH_HASHFUN_NAMESPACE": "std",
    "AXOM_MSVC_PRAGMAS": "",
}
ONES = {"AXOM_FMT_EXCEPTIONS": "1", "AXOM_FMT_HEADER_ONLY": "1"}


def _subst(text: str) -> str:
    out = []
    for line in text.splitlines():
        m = re.match(r"#cmakedefine01\s+(\w+)", line)
        if m:
            out.append(f"#define {m.group(1)} {ONES.get(m.group(1), '0')}")
            continue
        m = re.match(r"#cmakedefine\s+(\w+)(.*)", line)
        if m:
            name = m.group(1)
            out.append(f"#define {name}{m.group(2)}" if name in ENABLED else f"/* #undef {name} */")
            line = out.pop()
        line = re.sub(r"@(\w+)@", lambda mm: VALUES.get(mm.group(1), ""), line)
        out.append(line)
    return "\n".join(out) + "\n"


def _headers_of(ref_src: Path, comp: str) -> list[str]:
    cm = (ref_src / "axom" / comp / "CMakeLists.txt").read_text()
    m = re.search(r"set\(\s*%s_headers(.*?)\)" % comp, cm, re.S)
    names = re.findall(r"[\w/]+\.hpp", m.group(1)) if m else []
    return [n for n in names if "/detail/" not in f"/{n}" and "/internal/" not in f"/{n}"]


def generate(ref_src: Path) -> None:
    (GEN / "axom" / "export").mkdir(parents=True, exist_ok=True)
    (GEN / "axom" / "mint").mkdir(parents=True, exist_ok=True)
    (GEN / "axom" / "config.hpp").write_text(_subst((ref_src / "axom" / "config.hpp.in").read_text()))
    mint_cfg = (ref_src / "axom/mint/core/config.hpp.in").read_text()
    (GEN / "axom/mint/config.hpp").write_text(
        "\n".join(l for l in mint_cfg.splitlines() if not l.startswith("#cmakedefine")) + "\n")
    for comp in ("core", "slic", "mint", "primal", "spin", "quest", "slam", "sidre", "lumberjack"):
        (GEN / "axom/export" / f"{comp}.h").write_text(
            f"#ifndef AXOM_{comp.upper()}_EXPORT_H\n#define AXOM_{comp.upper()}_EXPORT_H\n"
            f"#define AXOM_{comp.upper()}_EXPORT\n#endif\n")
    for comp in UNIFIED:
        hdrs = _headers_of(ref_src, comp)
        if comp == "mint":
            hdrs = ["config.hpp"] + hdrs
        body = "".join(f'#include "axom/{comp}/{h}"\n' for h in hdrs)
        (GEN / "axom" / f"{comp}.hpp").write_text(
            f"#ifndef AXOM_UNIFIED_{comp.upper()}_HPP\n#define AXOM_UNIFIED_{comp.upper()}_HPP\n"
            f'#include "axom/config.hpp"\n{body}#endif\n')
    about = (ref_src / "axom/core/utilities/About.cpp.in").read_text()
    (GEN / "About.cpp").write_text(re.sub(r"@(\w+)@", "", about))


def _compile(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, p.returncode, p.stderr


def build(reference: Path, jobs: int) -> Path:
    ref_src = reference / "src"
    if not (ref_src / "axom/spin/BVH.hpp").exists():
        raise FileNotFoundError(f"reference sources not found under {ref_src}")
    generate(ref_src)
    OBJ.mkdir(parents=True, exist_ok=True)
    flags = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fopenmp",
             "-w", f"-I{GEN}", f"-I{ref_src}", f"-I{ref_src / 'thirdparty'}"]
    units = [(ref_src / s, OBJ / (s.replace("/", "_") + ".o")) for s in SOURCES]
    units.append((GEN / "About.cpp", OBJ / "About.o"))
    units.append((HERE / "ref_shim.cpp", OBJ / "ref_shim.o"))
    cmds = []
    for src, obj in units:
        if obj.exists() and obj.stat().st_mtime > src.stat().st_mtime:
            continue
        cmds.append(flags + ["-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for cmd, rc, err in ex.map(_compile, cmds):
            if rc != 0:
                raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{err[-4000:]}")
    link = ["g++", "-shared", "-fopenmp", "-o", str(LIB)] + [str(o) for _, o in units]
    p = subprocess.run(link, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stderr[-4000:]}")
    # keep only the library: the generated headers/objects are build by-products
    shutil.rmtree(GEN, ignore_errors=True)
    shutil.rmtree(OBJ, ignore_errors=True)
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=str(DEFAULT_REFERENCE))
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    print(build(Path(a.reference), a.j))
    return 0


if __name__ == "__main__":
    sys.exit(main())
