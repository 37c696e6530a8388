"""CPU: the oracle (C++ restatement) pinned against the reference and its tests.

* bit-exact against the committed golden fixtures (made by running the
  reference, tests/golden/make_golden.py);
* bit-exact against the reference library itself, live, where it is built;
* the reference's own known-answer tests (spin/tests/spin_bvh.cpp,
  quest/tests/quest_signed_distance.cpp, quest_signed_distance_interface.cpp).
"""
from __future__ import annotations

import numpy as np
import pytest

from axom_gb300 import workloads as W
from conftest import assert_bits_equal, golden

SCALES = [(1.000123, "s"), (1.0, "u")]


@pytest.mark.parametrize("scale,tag", SCALES)
def test_port_build_matches_golden(port, scale, tag):
    g = golden("bvh_boxes2000")
    it = port.internals(g["boxes"], scale)
    for k in ("codes", "perm", "lchild", "rchild", "parents", "inner", "bounds"):
        assert_bits_equal(it[k], g[f"{tag}_{k}"], k)


@pytest.mark.parametrize("scale,tag", SCALES)
def test_port_find_matches_golden(port, scale, tag):
    g = golden("bvh_boxes2000")
    h = port.bvh(g["boxes"], scale)
    assert_bits_equal(port.bounds(h), g[f"{tag}_bvh_bounds"], "bounds")
    for key, res in (("fb", port.find_boxes(h, g["query_boxes"])), ("fp", port.find_points(h, g["points"])),
                     ("fr", port.find_rays(h, g["ray_origins"], g["ray_dirs"]))):
        for name, arr in zip(("offsets", "counts", "candidates"), res):
            assert_bits_equal(arr, g[f"{tag}_{key}_{name}"], f"{key} {name}")


@pytest.mark.parametrize("scale,tag", SCALES)
def test_port_find_matches_dense_golden(port, scale, tag):
    """Candidate lists the reference made for queries that hit (18,721 box
    candidates, up to 99 per query; points inside and on the corners of
    boxes; rays aimed at boxes, some along the axes), order included."""
    g = golden("bvh_dense")
    h = port.bvh(g["boxes"], scale)
    assert_bits_equal(port.normalize_rays(g["ray_dirs_raw"]), g["ray_dirs"], "ray dirs")
    for key, res in (("fb", port.find_boxes(h, g["query_boxes"])), ("fp", port.find_points(h, g["points"])),
                     ("fr", port.find_rays(h, g["ray_origins"], g["ray_dirs"]))):
        for name, arr in zip(("offsets", "counts", "candidates"), res):
            assert_bits_equal(arr, g[f"{tag}_{key}_{name}"], f"{key} {name}")
    assert g[f"{tag}_fb_counts"].sum() > 15000


def test_port_ray_normalisation_matches_golden(port):
    g = golden("bvh_boxes2000")
    assert_bits_equal(port.normalize_rays(g["ray_dirs_raw"]), g["ray_dirs"], "ray dirs")


@pytest.mark.parametrize("name", ["sdf_uvsphere", "sdf_ico3", "sdf_ico3_open", "sdf_ico3_unsigned", "sdf_quad12"])
def test_port_sdf_matches_golden(port, name):
    g = golden(name)
    v = g["vertices"]
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], g["cells"], bool(g["watertight"]), bool(g["sign"]))
    d, cp, nr = port.sdf_eval(h, g["queries"], True, True)
    assert_bits_equal(d, g["dist"], "distance")
    assert_bits_equal(cp, g["closest"], "closest point")
    np.testing.assert_allclose(nr, g["normals"], rtol=0, atol=1e-12)
    assert_bits_equal(port.mesh_bounds(h), g["mesh_bounds"], "mesh bounds")
    if "box_tests" in g:
        nb, nl = port.sdf_counts(h, g["queries"])
        assert_bits_equal(nb, g["box_tests"], "box tests")
        assert_bits_equal(nl, g["leaf_tests"], "leaf tests")


def test_sphere_norms_match_reference_test():
    """quest_signed_distance.cpp:86-169: l1, l2, linf against the analytic sphere."""
    g = golden("sdf_uvsphere")
    phi = g["dist"]
    exact = np.linalg.norm(g["queries"], axis=1) - 0.5
    diff = phi - exact
    assert np.all(np.abs(diff) <= 1e-2)
    l1 = np.sum(np.abs(diff))
    l2 = np.sqrt(np.sum(diff))
    linf = np.max(np.abs(diff))
    assert abs(l1 - 6.7051997372579715) <= 1e-3
    assert abs(l2 - 2.5894400431865519) <= 1e-3
    assert abs(linf - 0.00532092) <= 1e-3


def _uniform_cells_3x3x3():
    return W.uniform_cells([0.0, 0.0, 0.0], [3.0, 3.0, 3.0], 4)


def test_known_answers_find_boxes(port):
    """spin_bvh.cpp:279-406: query box 0 hits cells 0-17, query box 1 hits none."""
    h = port.bvh(_uniform_cells_3x3x3(), 1.0)
    lo, hi = port.bounds(h)[:3], port.bounds(h)[3:]
    np.testing.assert_allclose(lo, 0.0, atol=1e-12)
    np.testing.assert_allclose(hi, 3.0, atol=1e-12)
    q = np.array([[-1.0, -1, -1, 2.5, 2.5, 1.5], [-1.0, -1, -1, -0.5, -0.5, -0.5]])
    off, cnt, cand = port.find_boxes(h, q)
    assert list(cnt) == [18, 0]
    assert sorted(cand[off[0]:off[0] + 18]) == list(range(18))


def test_known_answers_find_rays(port):
    """spin_bvh.cpp:519-648: the diagonal ray hits 15 listed cells, the opposite ray none."""
    h = port.bvh(_uniform_cells_3x3x3(), 1.0)
    o = np.array([[-1.0, -1, -1], [-1.0, -1, -1]])
    d = port.normalize_rays(np.array([[1.0, 1, 1], [-1.0, -1, -1]]))
    off, cnt, cand = port.find_rays(h, o, d)
    assert list(cnt) == [15, 0]
    assert sorted(cand) == [0, 1, 3, 4, 9, 10, 12, 13, 14, 16, 17, 22, 23, 25, 26]


def test_known_answers_find_points(port):
    """spin_bvh.cpp:792-903: each centroid hits exactly its cell; shifted points hit none."""
    cells = _uniform_cells_3x3x3()
    h = port.bvh(cells, 1.0)
    cent = 0.5 * (cells[:, :3] + cells[:, 3:])
    off, cnt, cand = port.find_points(h, cent)
    assert np.all(cnt == 1)
    assert np.array_equal(cand[off], np.arange(27))
    off, cnt, cand = port.find_points(h, cent + 10.0)
    assert np.all(cnt == 0)


def plane_mesh():
    """The 4-triangle open plane of quest_signed_distance_interface.cpp:61-108."""
    v = np.array([[-5.0, -5, 0], [5, -5, 0], [0, 0, 0], [5, 5, 0], [-5, 5, 0]])
    f = np.array([[0, 1, 2], [1, 3, 2], [3, 4, 2], [4, 0, 2]], np.int32)
    return v, f


def test_known_answers_plane(port):
    """quest_signed_distance_interface.cpp:186-242: exact distance to the plane z = 0."""
    v, f = plane_mesh()
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f, watertight=False)
    q = W.uniform_grid([-4.0] * 3, [4.0] * 3, 16)
    d, _, _ = port.sdf_eval(h, q)
    np.testing.assert_array_max_ulp(d, q[:, 2], maxulp=4)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 200])
def test_port_matches_reference_small(port, ref, n):
    boxes = W.random_boxes(n, 40 + n)
    if n >= 2:
        a, b = port.internals(boxes), ref.internals(boxes)
        for k in a:
            assert_bits_equal(a[k], b[k], k)
    hp, hr = port.bvh(boxes), ref.bvh(boxes)
    assert_bits_equal(port.bounds(hp), ref.bounds(hr), "bounds")
    q = W.random_boxes(300, 7)
    for x, y in zip(port.find_boxes(hp, q), ref.find_boxes(hr, q)):
        assert_bits_equal(x, y, "find boxes")


@pytest.mark.parametrize("scale", [1.000123, 1.0])
def test_port_matches_reference_config1(port, ref, scale):
    """The 100,000-box workload at its full size: boxes from seed 1, 100,000
    query boxes from seed 2 (centres U[0,1]^3, sides log-uniform in
    [1e-3, 1e-2]).  Morton codes, permutation, radix-tree links, parents,
    inner and leaf boxes, bounds, and the whole findBoundingBoxes CSR
    (candidate order included) against the reference's SEQ build."""
    boxes = W.random_boxes(100_000, 1)
    q = W.random_boxes(100_000, 2)
    a, b = port.internals(boxes, scale), ref.internals(boxes, scale)
    for k in a:
        assert_bits_equal(a[k], b[k], k)
    hp, hr = port.bvh(boxes, scale), ref.bvh(boxes, scale)
    assert_bits_equal(port.bounds(hp), ref.bounds(hr), "bounds")
    got, want = port.find_boxes(hp, q), ref.find_boxes(hr, q)
    for x, y, what in zip(got, want, ("offsets", "counts", "candidates")):
        assert_bits_equal(x, y, what)
    assert want[2].size > 4000
    # the threaded port (the CPU baseline's all-core form) gives the same CSR
    for x, y, what in zip(port.find_boxes_mt(hp, q, 7), want, ("offsets", "counts", "candidates")):
        assert_bits_equal(x, y, f"threaded {what}")
    # the find roofline's traversal counts, against the reference's own traverser
    assert_bits_equal(port.find_boxes_counts(hp, q[:20000]), ref.find_boxes_counts(hr, q[:20000]), "box tests")


def test_port_matches_reference_level8(port, ref):
    """The 1,310,720-triangle mesh of the signed-distance benchmark (level-8
    icosphere, seed 1234): the 20,000-point stratified sample of its 16M
    uniform points (seed 3) and 20,000 points within 1e-9..1e-3 of the surface.
    Distances, closest points and normals bit-exact against the reference,
    and the per-query box and triangle test counts of the uniform sample (the
    roofline numerator) equal to the reference traverser's."""
    v, f = W.displaced_icosphere(8, 1234)
    m = 1 << 24
    uni = W.uniform_queries(v, m, 3)[np.linspace(0, m - 1, 20000).astype(np.int64)]
    near = W.near_surface_queries(v, f, 20000, 4)
    q = np.concatenate([uni, near])
    hp = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    hr = ref.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    a = port.sdf_eval(hp, q, True, True, threads=8)
    b = ref.sdf_eval(hr, q, True, True, threads=8)
    for x, y, what in zip(a, b, ("distance", "closest", "normals")):
        assert_bits_equal(x, y, what)
    nbp, nlp = port.sdf_counts(hp, uni, threads=8)
    nbr, nlr = ref.sdf_counts(hr, uni, threads=8)
    assert_bits_equal(nbp, nbr, "box tests")
    assert_bits_equal(nlp, nlr, "triangle tests")


def test_port_matches_reference_edge_cases(port, ref):
    """Duplicate boxes (all Morton ties), invalid boxes, points as boxes, signed zeros."""
    rng = np.random.default_rng(3)
    dup = np.tile(W.random_boxes(1, 1), (64, 1))
    inval = W.random_boxes(50, 2)
    inval[::3, [0, 3]] = inval[::3, [3, 0]]  # min > max on x: invalid
    pts = rng.uniform(-1, 1, (40, 3))
    degen = np.concatenate([pts, pts], 1)
    zeros = np.zeros((8, 6))
    zeros[::2] = -0.0
    zeros[1::4, 3:] = 1.0
    nans = W.random_boxes(40, 4)
    nans[::5, 1] = np.nan  # a NaN coordinate: BoundingBox::isValid compares with ">", so still valid
    nans[2::5, 3] = np.nan
    nans[3::5, [0, 3]] = np.nan
    for boxes in (dup, inval, degen, zeros, nans, np.concatenate([dup, inval, degen, zeros, nans])):
        for scale in (1.000123, 1.0):
            a, b = port.internals(boxes, scale), ref.internals(boxes, scale)
            for k in a:
                assert_bits_equal(a[k], b[k], k)
            hp, hr = port.bvh(boxes, scale), ref.bvh(boxes, scale)
            q = np.concatenate([boxes[:20], W.random_boxes(20, 9) * 2 - 1])
            q[::7, 4] = np.nan
            for x, y in zip(port.find_boxes(hp, q), ref.find_boxes(hr, q)):
                assert_bits_equal(x, y, "find boxes")


def test_port_matches_reference_points_and_rays_edge_cases(port, ref):
    """findPoints with points on box corners, faces and inside, and findRays
    with axis-aligned directions (zero components: infinite slab parameters),
    zero directions, origins on corners and inside boxes, over boxes with
    duplicates, flat and invalid ones, at both scale factors."""
    rng = np.random.default_rng(11)
    lo = rng.uniform(0, 1, (300, 3))
    boxes = np.concatenate([lo, lo + rng.uniform(0, 0.25, (300, 3))], 1)
    boxes = np.concatenate([boxes, np.tile(boxes[:1], (16, 1))])
    boxes[::7, 2] = boxes[::7, 5]  # flat in z
    boxes[5::11, [1, 4]] = boxes[5::11, [4, 1]]  # invalid in y
    corners = np.concatenate([boxes[:60, :3], boxes[:60, 3:], np.stack([boxes[:60, 0], boxes[:60, 4],
                                                                       boxes[:60, 2]], 1)])
    faces = 0.5 * (boxes[:60, :3] + boxes[:60, 3:])
    faces[:, 0] = boxes[:60, 0]
    pts = np.concatenate([corners, faces, rng.uniform(-0.2, 1.2, (300, 3))])
    axes = np.repeat(np.eye(3), 20, axis=0) * np.where(rng.uniform(size=(60, 1)) < 0.5, -1.0, 1.0)
    dirs = np.concatenate([axes, np.zeros((5, 3)), rng.normal(size=(200, 3))])
    origins = np.concatenate([corners[: len(axes)], faces[:5], rng.uniform(-0.5, 1.5, (200, 3))])
    for scale in (1.000123, 1.0):
        hp, hr = port.bvh(boxes, scale), ref.bvh(boxes, scale)
        for x, y in zip(port.find_points(hp, pts), ref.find_points(hr, pts)):
            assert_bits_equal(x, y, f"find points, scale {scale}")
        *got, unit = ref.find_rays(hr, origins, dirs)
        assert_bits_equal(port.normalize_rays(dirs), unit, "ray normalisation")
        for x, y in zip(port.find_rays(hp, origins, unit), got):
            assert_bits_equal(x, y, f"find rays, scale {scale}")
        assert got[1].sum() > 100 and (got[1] == 0).any()  # hits and misses


def test_port_matches_reference_sdf_live(port, ref):
    v, f = W.displaced_icosphere(4, 77)
    q = W.mixed_queries(v, f, 3000, 5)
    for wt, sg in ((True, True), (False, True), (True, False)):
        hp = port.sdf(v[:, 0], v[:, 1], v[:, 2], f, wt, sg)
        hr = ref.sdf(v[:, 0], v[:, 1], v[:, 2], f, wt, sg)
        a = port.sdf_eval(hp, q, True, True)
        b = ref.sdf_eval(hr, q, True, True)
        assert_bits_equal(a[0], b[0], "distance")
        assert_bits_equal(a[1], b[1], "closest")
        assert_bits_equal(a[2], b[2], "normals")


def _on_features(v, f):
    """Points exactly on vertices, edge midpoints and centroids of the cells."""
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    return np.concatenate([v, 0.5 * (a + b), 0.5 * (b + c), (a + b + c) / 3.0])


@pytest.mark.parametrize("case", ["slivers", "quads", "tiny1", "tiny2", "empty"])
def test_port_matches_reference_sdf_edge_cases(port, ref, case):
    """Slivers and zero-area triangles (open surface), quad cells, meshes of
    0, 1 and 2 triangles (BVH padding; an empty mesh gives sqrt(DBL_MAX)),
    points exactly on vertices, edges and faces and far away, every
    watertight / sign combination."""
    if case == "slivers":
        v, f = W.sliver_sheet(3)
    elif case == "quads":
        v, f = W.quad_sphere(12)
        v = W.displace(v, 8)
    else:
        v = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.5]])
        f = {"tiny1": [[0, 1, 2]], "tiny2": [[0, 1, 2], [1, 3, 2]], "empty": np.zeros((0, 3))}[case]
        f = np.asarray(f, np.int32)
    pts = [W.uniform_queries(v, 2000, 1), W.uniform_queries(v, 200, 2, factor=40.0)]
    if f.shape[0]:
        pts.append(_on_features(v, f[:, :3])[:: max(1, v.shape[0] // 500)])
    q = np.concatenate(pts)
    for wt, sg in ((True, True), (False, True), (True, False), (False, False)):
        hp = port.sdf(v[:, 0], v[:, 1], v[:, 2], f, wt, sg)
        hr = ref.sdf(v[:, 0], v[:, 1], v[:, 2], f, wt, sg)
        a = port.sdf_eval(hp, q, True, True)
        b = ref.sdf_eval(hr, q, True, True)
        for x, y, what in zip(a, b, ("distance", "closest", "normals")):
            assert_bits_equal(x, y, f"{case} {what} (watertight {wt}, sign {sg})")


@pytest.mark.parametrize("tag", ["all", "thr"])
def test_port_closest_point_matches_golden(port, tag):
    """DistributedClosestPoint's local query against the reference's outputs."""
    g = golden("cp_points3000")
    thr = float(np.finfo(np.float64).max) if tag == "all" else 0.05 * 0.05
    h = port.cp(g["points"], g["domains"])
    idx, dom, pos, dist = port.cp_query(h, g["queries"], thr, threads=4)
    assert_bits_equal(idx, g[f"{tag}_idx"], "index")
    assert_bits_equal(dom, g[f"{tag}_dom"], "domain")
    assert_bits_equal(pos, g[f"{tag}_pos"], "position")
    assert_bits_equal(dist, g[f"{tag}_dist"], "distance")


@pytest.mark.parametrize("n", [0, 1, 2, 5000])
def test_port_closest_point_matches_reference_live(port, ref, n):
    """Empty and one-point clouds (padded trees), ties from duplicate points,
    points on the queries, a threshold."""
    r = np.random.default_rng(30 + n)
    pts = r.uniform(0, 1, (n, 3))
    if n > 2:
        pts[n // 2:] = pts[: n - n // 2]
    dom = r.integers(0, 9, n).astype(np.int32)
    q = r.uniform(-0.3, 1.3, (4000, 3))
    if n:
        q[: min(n, 100)] = pts[: min(n, 100)]
    hp, hr = port.cp(pts, dom), ref.cp(pts, dom)
    for thr in (float(np.finfo(np.float64).max), 0.01):
        for x, y, what in zip(port.cp_query(hp, q, thr, threads=4), ref.cp_query(hr, q, thr, threads=4),
                              ("index", "domain", "position", "distance")):
            assert_bits_equal(x, y, what)


def test_port_threads_are_deterministic(port):
    v, f = W.displaced_icosphere(3, 1)
    q = W.uniform_queries(v, 4000, 2)
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    a = port.sdf_eval(h, q, threads=1)[0]
    b = port.sdf_eval(h, q, threads=4)[0]
    assert_bits_equal(a, b, "threads")
