"""CPU: the STL reader (quest::STLReader) of the library against the
reference's own reader, on ASCII and binary files written here.

Host code only (no GPU); bit-exact coordinates and connectivity."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from axom_gb300 import workloads as W
from conftest import assert_bits_equal


@pytest.fixture(scope="module")
def lib():
    from axom_gb300 import build
    build.build()
    import axom_gb300
    return axom_gb300


def write_ascii(path, tris, fmt="{:.17g}"):
    with open(path, "w") as f:
        f.write("solid test\n")
        for t in tris:
            f.write("  facet normal 0 0 1\n    outer loop\n")
            for p in t:
                f.write("      vertex " + " ".join(fmt.format(c) for c in p) + "\n")
            f.write("    endloop\n  endfacet\n")
        f.write("endsolid test\n")


def write_binary(path, tris):
    with open(path, "wb") as f:
        f.write(b"binary stl".ljust(80, b"\0"))
        f.write(struct.pack("<i", len(tris)))
        for t in tris:
            f.write(struct.pack("<12fH", 0.0, 0.0, 1.0, *np.asarray(t, np.float32).ravel(), 0))


def mesh_tris(level=2, seed=3):
    v, f = W.displaced_icosphere(level, seed)
    return v[f]


def test_ascii_and_binary_round_trip(lib, tmp_path):
    tris = mesh_tris()
    write_ascii(tmp_path / "a.stl", tris)
    v, f = lib.read_stl(tmp_path / "a.stl")
    assert_bits_equal(v, tris.reshape(-1, 3), "ascii coordinates")
    assert np.array_equal(f, np.arange(3 * len(tris)).reshape(-1, 3))
    write_binary(tmp_path / "b.stl", tris)
    v, f = lib.read_stl(tmp_path / "b.stl")
    assert_bits_equal(v, tris.reshape(-1, 3).astype(np.float32).astype(np.float64), "binary coordinates")


@pytest.mark.parametrize("kind", ["ascii17", "ascii_sci", "ascii_short", "binary", "empty", "partial"])
def test_matches_reference_reader(lib, ref, tmp_path, kind):
    tris = mesh_tris(3, 5) * 37.5 - 3.0
    p = tmp_path / f"{kind}.stl"
    if kind == "ascii17":
        write_ascii(p, tris)
    elif kind == "ascii_sci":
        write_ascii(p, tris, "{:.9E}")
    elif kind == "ascii_short":
        write_ascii(p, tris, "{:.3f}")
    elif kind == "binary":
        write_binary(p, tris)
    elif kind == "empty":
        p.write_text("solid nothing\nendsolid nothing\n")
    else:  # seven vertices: two full triangles and a stray node
        write_ascii(p, tris[:3])
        text = p.read_text().splitlines()
        p.write_text("\n".join(text[:-5]) + "\n")  # the third facet keeps one vertex
    want = ref.stl_read(p)
    got = lib.read_stl(p)
    assert want is not None
    assert_bits_equal(got[0], want[0], "coordinates")
    assert np.array_equal(got[1], want[1])


def test_missing_file_is_an_error(lib, tmp_path):
    with pytest.raises(lib.GsqError):
        lib.read_stl(tmp_path / "does_not_exist.stl")
