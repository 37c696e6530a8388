"""GPU: signed distance through the C ABI against the oracle and the golden
fixtures.  The FP64 form is bit-exact in distance and closest point; unit
normals are checked to 1e-12 (they go through acos, whose last bit may differ
between CUDA's and the host's libm)."""
from __future__ import annotations

import numpy as np
import pytest

import axom_gb300
from axom_gb300 import workloads as W
from conftest import assert_bits_equal, golden

pytestmark = pytest.mark.gpu

NORMAL_ATOL = 1e-12
FIXTURES = ["sdf_uvsphere", "sdf_ico3", "sdf_ico3_open", "sdf_ico3_unsigned", "sdf_quad12"]


def make(gsq, g, **kw):
    return gsq.SignedDistance(g["vertices"], g["cells"], bool(g["watertight"]), bool(g["sign"]), **kw)


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("sort_queries", [True, False])
def test_fp64_matches_golden(gsq, name, sort_queries):
    g = golden(name)
    sd = make(gsq, g, sort_queries=sort_queries)
    d, cp, nr = sd.compute_distances(g["queries"], closest=True, normals=True)
    assert_bits_equal(d, g["dist"], "distance")
    assert_bits_equal(cp, g["closest"], "closest point")
    np.testing.assert_allclose(nr, g["normals"], rtol=0, atol=NORMAL_ATOL)
    lo, hi = sd.get_mesh_bounds()
    assert_bits_equal(np.concatenate([lo, hi]), g["mesh_bounds"], "mesh bounds")


def test_sphere_norms(gsq):
    g = golden("sdf_uvsphere")
    phi = make(gsq, g).compute_distances(g["queries"])
    diff = phi - (np.linalg.norm(g["queries"], axis=1) - 0.5)
    assert abs(np.sum(np.abs(diff)) - 6.7051997372579715) <= 1e-3
    assert abs(np.sqrt(np.sum(diff)) - 2.5894400431865519) <= 1e-3
    assert abs(np.max(np.abs(diff)) - 0.00532092) <= 1e-3


def test_plane_exact(gsq):
    v = np.array([[-5.0, -5, 0], [5, -5, 0], [0, 0, 0], [5, 5, 0], [-5, 5, 0]])
    f = np.array([[0, 1, 2], [1, 3, 2], [3, 4, 2], [4, 0, 2]], np.int32)
    sd = gsq.SignedDistance(v, f, is_watertight=False)
    q = W.uniform_grid([-4.0] * 3, [4.0] * 3, 16)
    np.testing.assert_array_max_ulp(sd.compute_distances(q), q[:, 2], maxulp=4)


def test_layouts_and_memory_spaces_agree(gsq):
    import torch
    g = golden("sdf_ico3")
    sd = make(gsq, g)
    q = g["queries"]
    ref = sd.compute_distances(q)
    dev = sd.compute_distances(torch.from_numpy(q).cuda()).cpu().numpy()
    assert_bits_equal(dev, g["dist"], "device AoS")
    qx, qy, qz = (np.ascontiguousarray(q[:, k]) for k in range(3))
    out = np.empty(q.shape[0])
    sd.compute_distances_soa(qx, qy, qz, out)
    assert_bits_equal(out, ref, "SoA")
    assert sd.compute_distance(*q[7]) == ref[7]


@pytest.mark.parametrize("level,m", [(5, 30000), (6, 20000)])
def test_fp64_matches_oracle_random(gsq, port, level, m):
    v, f = W.displaced_icosphere(level, 99 + level)
    q = W.mixed_queries(v, f, m, level)
    sd = gsq.SignedDistance(v, f)
    d, cp, nr = sd.compute_distances(q, closest=True, normals=True)
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    pd, pcp, pnr = port.sdf_eval(h, q, True, True, threads=8)
    assert_bits_equal(d, pd, "distance")
    assert_bits_equal(cp, pcp, "closest")
    np.testing.assert_allclose(nr, pnr, rtol=0, atol=NORMAL_ATOL)


def test_tiny_meshes(gsq, port):
    """0, 1 and 2 triangles (BVH padding), one point query far away and near."""
    v = np.array([[0.0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0.5]])
    q = np.array([[0.2, 0.2, 0.3], [5.0, -3, 2], [0.5, 0.5, -0.1], [0.0, 0.0, 0.0]])
    for f in (np.zeros((0, 3), np.int32), np.array([[0, 1, 2]], np.int32),
              np.array([[0, 1, 2], [1, 3, 2]], np.int32)):
        for wt in (True, False):
            h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f, wt, True)
            pd, pcp, _ = port.sdf_eval(h, q, True, True)
            for precision in (axom_gb300.PRECISION_FP64, axom_gb300.PRECISION_MIXED):
                sd = gsq.SignedDistance(v, f, is_watertight=wt, precision=precision)
                d, cp, _ = sd.compute_distances(q, closest=True, normals=True)
                assert_bits_equal(d, pd, "distance")
                assert_bits_equal(cp, pcp, "closest")
                assert sd.compute_distances(q[:0]).shape == (0,)  # no points


def test_full_size_sample(gsq, port):
    """Level-8 displaced icosphere (1,310,720 triangles) with 16M uniform
    queries on the GPU; a 20,000-point stratified sample against the oracle,
    and the whole output for finiteness and inside fraction."""
    import torch
    v, f = W.displaced_icosphere(8, 1234)
    m = 1 << 24
    q = torch.from_numpy(W.uniform_queries(v, m, 3)).cuda()
    sd = gsq.SignedDistance(v, f)
    d = sd.compute_distances(q).cpu().numpy()
    assert np.all(np.isfinite(d))
    inside = np.mean(d < 0)
    assert 0.15 < inside < 0.30
    idx = np.linspace(0, m - 1, 20000).astype(np.int64)
    qs = q[idx].cpu().numpy()
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    pd, _, _ = port.sdf_eval(h, qs, threads=16)
    assert_bits_equal(d[idx], pd, "distance sample")


def test_concurrent_calls_on_one_handle(gsq):
    """computeDistances and the BVH's find* are const and re-entrant in the
    reference: four host threads, each on its own stream, evaluate (mixed
    form) and find on one shared handle at the same time; every result equals
    the single-threaded one bit for bit."""
    import threading
    import torch
    v, f = W.displaced_icosphere(5, 3)
    q = torch.from_numpy(W.mixed_queries(v, f, 200_000, 4)).cuda()
    sd = gsq.SignedDistance(v, f, precision=gsq.PRECISION_MIXED)
    want = sd.compute_distances(q)
    boxes = W.random_boxes(50_000, 5)
    qb = torch.from_numpy(W.random_boxes(50_000, 6) * 1.5 - 0.25).cuda()
    bvh = gsq.BVH(boxes)
    want_f = [x.cpu().numpy() for x in bvh.find_bounding_boxes(qb)]
    errors = []

    def work(k):
        try:
            st = torch.cuda.Stream()
            with torch.cuda.stream(st):
                for _ in range(3):
                    d = sd.compute_distances(q)
                    got_f = bvh.find_bounding_boxes(qb)
                    st.synchronize()
                    if not torch.equal(d.view(torch.int64), want.view(torch.int64)):
                        errors.append(f"thread {k}: distances differ")
                    for x, y in zip(got_f, want_f):
                        if not np.array_equal(x.cpu().numpy(), y):
                            errors.append(f"thread {k}: candidates differ")
        except Exception as e:  # reported below
            errors.append(f"thread {k}: {e!r}")

    threads = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors[:4]
