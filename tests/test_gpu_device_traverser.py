"""GPU: user kernels traverse a gsq BVH through include/gsq_device.cuh
(the getTraverser role, spin/BVH.hpp:319).  A two-pass point query written
against the header (tests/cpp/two_pass.cu, compiled here with nvcc) must give
the same counts and the same candidates in the same order as the oracle's
findPoints (and so gsq_bvh_find_points)."""
from __future__ import annotations

import ctypes as C
import subprocess

import numpy as np
import pytest

from axom_gb300 import workloads as W
from conftest import ROOT, assert_bits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def two_pass(tmp_path_factory):
    from axom_gb300 import build
    so = tmp_path_factory.mktemp("two_pass") / "libtwo_pass.so"
    subprocess.run([build.nvcc(), *build.ARCH, "-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                    "-shared", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/two_pass.cu"), "-o", str(so)],
                   check=True)
    lib = C.CDLL(str(so))
    for f in (lib.two_pass_count, lib.two_pass_fill):
        f.restype = C.c_int
    return lib


def test_user_kernel_matches_find_points(gsq, port, two_pass):
    import torch
    boxes = W.random_boxes(100_000, 3)
    r = W.rng(4)
    pts = r.uniform(0, 1, (50_000, 3))
    pick = r.integers(0, len(boxes), 25_000)  # half of the points inside a box
    pts[::2] = boxes[pick, :3] + r.uniform(0, 1, (25_000, 3)) * (boxes[pick, 3:] - boxes[pick, :3])
    bvh = gsq.BVH(boxes)
    view = bvh.get_view()
    assert view.num_leaves == 100_000
    p = torch.from_numpy(pts).cuda()
    counts = torch.empty(len(pts), dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert two_pass.two_pass_count(C.byref(view), C.c_void_p(p.data_ptr()), len(pts), C.c_void_p(counts.data_ptr()),
                                   C.c_void_p(err.data_ptr())) == 0
    assert int(err.item()) == 0
    offsets = torch.zeros(len(pts), dtype=torch.int32, device="cuda")
    offsets[1:] = torch.cumsum(counts, 0)[:-1].to(torch.int32)
    cands = torch.empty(max(int(counts.sum().item()), 1), dtype=torch.int32, device="cuda")
    assert two_pass.two_pass_fill(C.byref(view), C.c_void_p(p.data_ptr()), len(pts), C.c_void_p(offsets.data_ptr()),
                                  C.c_void_p(cands.data_ptr())) == 0
    off, cnt, cand = port.find_points(port.bvh(boxes), pts)
    assert cand.size > 25_000
    assert_bits_equal(counts.cpu().numpy(), cnt, "counts")
    assert_bits_equal(offsets.cpu().numpy(), off, "offsets")
    assert_bits_equal(cands.cpu().numpy()[: len(cand)], cand, "candidates")
    for x, y, what in zip(bvh.find_points(pts), (off, cnt, cand), ("offsets", "counts", "candidates")):
        assert_bits_equal(np.asarray(x), y, f"gsq_bvh_find_points {what}")
