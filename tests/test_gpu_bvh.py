"""GPU: BVH build and candidate queries through the C ABI, bit-exact against
the oracle and the golden fixtures made by the reference."""
from __future__ import annotations

import numpy as np
import pytest

from axom_gb300 import workloads as W
from conftest import assert_bits_equal, golden

pytestmark = pytest.mark.gpu


def check_layout(gsq, port, boxes, scale):
    b = gsq.BVH(boxes, scale_factor=scale)
    h = port.bvh(boxes, scale)
    nodes, ch, leaf, codes = b.export()
    pn, pc, pl = port.layout(h)
    assert_bits_equal(leaf, pl, "leaf ids")
    assert_bits_equal(ch, pc, "children")
    assert_bits_equal(nodes, pn, "node boxes")
    lo, hi = b.get_bounds()
    assert_bits_equal(np.concatenate([lo, hi]), port.bounds(h), "bounds")
    return b, h


@pytest.mark.parametrize("scale,tag", [(1.000123, "s"), (1.0, "u")])
def test_build_matches_golden(gsq, scale, tag):
    g = golden("bvh_boxes2000")
    b = gsq.BVH(g["boxes"], scale_factor=scale)
    nodes, ch, leaf, codes = b.export()
    assert_bits_equal(codes, g[f"{tag}_codes"], "codes")
    assert_bits_equal(leaf, g[f"{tag}_perm"], "permutation")
    lo, hi = b.get_bounds()
    assert_bits_equal(np.concatenate([lo, hi]), g[f"{tag}_bounds"], "bounds")
    # children in the reference's encoding, rebuilt from the radix-tree links
    n = g["boxes"].shape[0]
    inner = n - 1
    enc = lambda c: np.where(c >= inner, -(c - inner + 1), 2 * c)  # noqa: E731
    exp = np.stack([enc(g[f"{tag}_lchild"]), enc(g[f"{tag}_rchild"])], 1).reshape(-1)
    assert_bits_equal(ch, exp.astype(np.int32), "children")


@pytest.mark.parametrize("scale,tag", [(1.000123, "s"), (1.0, "u")])
def test_find_matches_golden(gsq, scale, tag):
    g = golden("bvh_boxes2000")
    b = gsq.BVH(g["boxes"], scale_factor=scale)
    for key, res in (("fb", b.find_bounding_boxes(g["query_boxes"])), ("fp", b.find_points(g["points"])),
                     ("fr", b.find_rays(g["ray_origins"], g["ray_dirs"]))):
        for name, arr in zip(("offsets", "counts", "candidates"), res):
            assert_bits_equal(arr, g[f"{tag}_{key}_{name}"], f"{key} {name}")


@pytest.mark.parametrize("scale,tag", [(1.000123, "s"), (1.0, "u")])
def test_find_matches_dense_golden(gsq, scale, tag):
    """The reference's candidate lists for queries that hit: 18,721 box
    candidates (up to 99 per query), points inside and on box corners, rays
    aimed at boxes and along the axes; offsets, counts and candidate order."""
    g = golden("bvh_dense")
    b = gsq.BVH(g["boxes"], scale_factor=scale)
    for key, res in (("fb", b.find_bounding_boxes(g["query_boxes"])), ("fp", b.find_points(g["points"])),
                     ("fr", b.find_rays(g["ray_origins"], g["ray_dirs"]))):
        for name, arr in zip(("offsets", "counts", "candidates"), res):
            assert_bits_equal(arr, g[f"{tag}_{key}_{name}"], f"{key} {name}")


@pytest.mark.parametrize("scale", [1.000123, 1.0])
def test_config1_full_size_matches_oracle(gsq, port, scale):
    """The 100,000-box workload at its full size: 100,000 boxes (seed 1),
    100,000 query boxes (seed 2).  Morton codes, permutation, children, node
    boxes and bounds, and the whole findBoundingBoxes CSR, bit-exact against
    the oracle (itself pinned to the reference at this size on the CPU)."""
    boxes = W.random_boxes(100_000, 1)
    q = W.random_boxes(100_000, 2)
    b, h = check_layout(gsq, port, boxes, scale)
    assert_bits_equal(b.export()[3], port.internals(boxes, scale)["codes"], "codes")
    got = b.find_bounding_boxes(q)
    want = port.find_boxes(h, q)
    for x, y, what in zip(got, want, ("offsets", "counts", "candidates")):
        assert_bits_equal(x, y, what)
    assert want[2].size > 4000


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 17, 100, 1023, 1024, 1025, 3000, 4095, 4096, 4097, 50000])
def test_build_sizes_match_oracle(gsq, port, n):
    boxes = W.random_boxes(n, 100 + n) if n else np.zeros((0, 6))
    b, h = check_layout(gsq, port, boxes, 1.000123)
    q = W.random_boxes(2000, 3)
    for x, y in zip(b.find_bounding_boxes(q), port.find_boxes(h, q)):
        assert_bits_equal(x, y, "find boxes")


def test_build_edge_cases_match_oracle(gsq, port):
    rng = np.random.default_rng(3)
    dup = np.tile(W.random_boxes(1, 1), (5000, 1))
    inval = W.random_boxes(3000, 2)
    inval[::3, [0, 3]] = inval[::3, [3, 0]]
    pts = rng.uniform(-1, 1, (2000, 3))
    degen = np.concatenate([pts, pts], 1)
    zeros = np.zeros((64, 6))
    zeros[::2] = -0.0
    zeros[1::4, 3:] = 1.0
    allinv = np.tile(np.array([[1.0, 1, 1, 0, 0, 0]]), (10, 1))
    nans = W.random_boxes(3000, 4)
    nans[::5, 1] = np.nan  # still valid for BoundingBox::isValid, which compares with ">"
    nans[2::5, 3] = np.nan
    nans[3::5, [0, 3]] = np.nan
    for boxes in (dup, inval, degen, zeros, allinv, nans, np.concatenate([dup, inval, degen, zeros, nans])):
        for scale in (1.000123, 1.0):
            b, h = check_layout(gsq, port, boxes, scale)
            q = np.concatenate([boxes[:200], W.random_boxes(200, 9) * 2 - 1])
            q[::7, 4] = np.nan
            for x, y in zip(b.find_bounding_boxes(q), port.find_boxes(h, q)):
                assert_bits_equal(x, y, "find boxes")


def test_find_points_and_rays_match_oracle(gsq, port):
    boxes = W.random_boxes(20000, 8)
    b, h = check_layout(gsq, port, boxes, 1.000123)
    p = W.rng(4).uniform(0, 1, (20000, 3))
    p[::11, 2] = np.nan
    for x, y in zip(b.find_points(p), port.find_points(h, p)):
        assert_bits_equal(x, y, "find points")
    o = W.rng(5).uniform(-0.5, 1.5, (3000, 3))
    d = port.normalize_rays(W.rng(6).normal(size=(3000, 3)))
    d[::5, 1] = 0.0
    o[::13, 0] = np.nan
    d[::17, 2] = np.nan
    for x, y in zip(b.find_rays(o, d), port.find_rays(h, o, d)):
        assert_bits_equal(x, y, "find rays")


def test_known_answers(gsq):
    cells = W.uniform_cells([0.0] * 3, [3.0] * 3, 4)
    b = gsq.BVH(cells, scale_factor=1.0)
    off, cnt, cand = b.find_bounding_boxes(np.array([[-1.0, -1, -1, 2.5, 2.5, 1.5], [-1.0, -1, -1, -0.5, -0.5, -0.5]]))
    assert list(cnt) == [18, 0] and sorted(cand) == list(range(18))
    d = gsq.normalize_rays(np.array([[1.0, 1, 1], [-1.0, -1, -1]]))
    off, cnt, cand = b.find_rays(np.array([[-1.0, -1, -1]] * 2), d)
    assert list(cnt) == [15, 0]
    assert sorted(cand) == [0, 1, 3, 4, 9, 10, 12, 13, 14, 16, 17, 22, 23, 25, 26]
    cent = 0.5 * (cells[:, :3] + cells[:, 3:])
    off, cnt, cand = b.find_points(cent)
    assert np.all(cnt == 1) and np.array_equal(cand[off], np.arange(27))
    off, cnt, cand = b.find_points(cent + 10.0)
    assert np.all(cnt == 0) and cand.size == 0


def test_device_and_host_buffers_agree(gsq):
    import torch
    boxes = W.random_boxes(30000, 12)
    q = W.random_boxes(30000, 13) * 1.05
    bh = gsq.BVH(boxes)
    bd = gsq.BVH(torch.from_numpy(boxes).cuda())
    for x, y in zip(bh.find_bounding_boxes(q), bd.find_bounding_boxes(torch.from_numpy(q).cuda())):
        assert_bits_equal(x, y.cpu().numpy(), "host vs device")


def test_many_candidates_overflow_path(gsq, port):
    """Queries with far more candidates than the per-query scratch keeps."""
    boxes = W.random_boxes(5000, 21)
    q = np.array([[0.0, 0, 0, 1, 1, 1], [0.2, 0.2, 0.2, 0.6, 0.6, 0.6], [0.5, 0.5, 0.5, 0.5, 0.5, 0.5]])
    b, h = check_layout(gsq, port, boxes, 1.000123)
    for x, y in zip(b.find_bounding_boxes(q), port.find_boxes(h, q)):
        assert_bits_equal(x, y, "find boxes")


def test_full_size_triangle_boxes_build(gsq, port):
    """1,310,720 triangle boxes of the level-8 icosphere: build bit-exact."""
    v, f = W.displaced_icosphere(8, 1234)
    tri = v[f]
    boxes = np.concatenate([tri.min(1), tri.max(1)], 1)
    check_layout(gsq, port, boxes, 1.000123)


def test_mesh_self_query_broad_phase(gsq, port):
    """The broad phase of MeshTester's self-intersection test
    (quest/detail/MeshTester_detail.hpp:320-340): findBoundingBoxes with a
    mesh's own triangle boxes as the queries (81,920 triangles, every box
    touching its neighbours); the candidate CSR equals the oracle's."""
    v, f = W.displaced_icosphere(6, 5)
    tri = v[f]
    boxes = np.concatenate([tri.min(1), tri.max(1)], 1)
    b, h = check_layout(gsq, port, boxes, 1.000123)
    got, want = b.find_bounding_boxes(boxes), port.find_boxes(h, boxes)
    for x, y in zip(got, want):
        assert_bits_equal(x, y, "self query")
    assert int(got[1].min()) >= 1  # every box finds at least itself


def test_rebuilt_handle_answers_for_its_new_boxes(gsq, port):
    """One handle rebuilt over other boxes (other counts, then the same count
    with other coordinates, then the first set again, which replays the
    captured build) answers box, point and ray finds for the boxes it holds:
    the per-node key records of the box and point finds are remade after every
    build."""
    sets = [W.random_boxes(30_000, 31), W.random_boxes(12_000, 32), W.random_boxes(12_000, 33),
            W.random_boxes(30_000, 31), W.random_boxes(30_000, 31)]
    q = W.random_boxes(3_000, 34)
    r = W.rng(35)
    pts = r.uniform(0, 1, (3_000, 3))
    o = r.uniform(-0.1, 1.1, (500, 3))
    d = port.normalize_rays(r.normal(size=(500, 3)))
    b = gsq.BVH()
    for boxes in sets:
        b.initialize(boxes)
        h = port.bvh(boxes)
        for x, y in zip(b.find_bounding_boxes(q), port.find_boxes(h, q)):
            assert_bits_equal(np.asarray(x), y, "find boxes after a rebuild")
        for x, y in zip(b.find_points(pts), port.find_points(h, pts)):
            assert_bits_equal(np.asarray(x), y, "find points after a rebuild")
        for x, y in zip(b.find_rays(o, d), port.find_rays(h, o, d)):
            assert_bits_equal(np.asarray(x), y, "find rays after a rebuild")
