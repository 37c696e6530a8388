"""GPU: the batched form (many meshes and point sets, one CUDA graph per run).

Every mesh's distances and closest points must equal a standalone
SignedDistance of that mesh (itself pinned to the reference) bit for bit:
the segmented build must give each mesh the tree a standalone build gives it,
and the shared persistent query must evaluate each point against its own
mesh.  Tolerance: bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import axom_gb300
from axom_gb300 import workloads as W
from conftest import assert_bits_equal

pytestmark = pytest.mark.gpu


def small_batch(n, seed, levels=(2, 4), points=(1_000, 20_000), near=True, quads=False):
    """n transformed icospheres (or quad spheres), uniform points in each
    expanded box plus points near the surface."""
    r = np.random.default_rng(seed)
    meshes, pts = W.batch_meshes(n, seed, levels=levels, points=points)
    if quads:
        meshes = []
        for k in range(n):
            v, f = W.quad_sphere(int(r.integers(4, 12)))
            v = (v @ W.random_rotation(r).T) * r.uniform(0.5, 2.0) + r.uniform(-10, 10, size=3)
            meshes.append((v, f))
        pts = [W.uniform_queries(v, int(r.integers(500, 5000)), seed + k) for k, (v, _) in enumerate(meshes)]
    if near and not quads:
        pts = [np.concatenate([p, W.near_surface_queries(v, f, max(64, p.shape[0] // 4), seed + 31 * k)])
               for k, ((v, f), p) in enumerate(zip(meshes, pts))]
    return meshes, pts


def standalone(meshes, pts, watertight=True, sign=True, closest=True):
    res = []
    for (v, f), p in zip(meshes, pts):
        sd = axom_gb300.SignedDistance(v, f, is_watertight=watertight, compute_sign=sign,
                                       precision=axom_gb300.PRECISION_FP64)
        if closest:
            d, cp, _ = sd.compute_distances(p, closest=True)
            res.append((d, cp))
        else:
            res.append((sd.compute_distances(p), None))
    return res


def check(batch, flat_d, flat_cp, expect):
    for k, (dk, ck) in enumerate(zip(batch.split(flat_d), batch.split(flat_cp) if flat_cp is not None
                                     else [None] * len(expect))):
        d_ref, cp_ref = expect[k]
        assert_bits_equal(dk, d_ref, f"mesh {k} distance")
        if ck is not None:
            assert_bits_equal(ck, cp_ref, f"mesh {k} closest point")


@pytest.mark.parametrize("watertight,sign", [(True, True), (False, True), (True, False)])
def test_batch_equals_standalone(gsq, watertight, sign):
    meshes, pts = small_batch(24, 11)
    if not watertight:
        meshes = [(v, f[np.arange(f.shape[0]) % 7 != 3]) for v, f in meshes]
    b = gsq.Batch(meshes, pts, is_watertight=watertight, compute_sign=sign, closest_points=True)
    d, cp = b.run(closest=True)
    check(b, d, cp, standalone(meshes, pts, watertight, sign))
    # a second replay of the same graph gives the same bits
    d2 = b.run()
    assert_bits_equal(d2, d, "replay")


def test_batch_quads(gsq):
    meshes, pts = small_batch(12, 5, quads=True)
    b = gsq.Batch(meshes, pts, closest_points=True)
    d, cp = b.run(closest=True)
    check(b, d, cp, standalone(meshes, pts))


def test_batch_rebuilds_from_new_vertices(gsq):
    """Coordinates change between runs; each run rebuilds every tree."""
    meshes, pts = small_batch(16, 3)
    b = gsq.Batch(meshes, pts)
    b.run()
    r = np.random.default_rng(8)
    moved = [(v * r.uniform(0.8, 1.2) + r.uniform(-1, 1, size=3), f) for v, f in meshes]
    b.set_vertices(np.concatenate([v for v, _ in moved]))
    d = b.run()
    check(b, d, None, standalone(moved, pts, closest=False))


def test_batch_device_points_and_empty_sets(gsq):
    import torch
    meshes, pts = small_batch(10, 21)
    pts[3] = pts[3][:0]  # a mesh with no points
    pts[7] = pts[7][:1]
    b = gsq.Batch(meshes, [torch.from_numpy(p).cuda() for p in pts])
    out = torch.empty(b.num_points, dtype=torch.float64, device="cuda")
    b.run(out=out)
    expect = [(e[0], None) for e in standalone(meshes, pts, closest=False)]
    check(b, out.cpu().numpy(), None, expect)


def host_max_depth(v, f):
    """Deepest leaf (edges from the root) of the standalone tree of one mesh,
    from its exported child links (inner child c at node c // 2, leaves < 0)."""
    sd = axom_gb300.SignedDistance(v, f)
    _, children, _, _ = sd.get_bvh_tree().export()
    children = children.reshape(-1, 2)
    best = 0
    stack = [(0, 0)]
    while stack:
        node, d = stack.pop()
        for c in children[node]:
            if c >= 0:
                stack.append((int(c) // 2, d + 1))
            else:
                best = max(best, d + 1)
    return best


def test_batch_tune(gsq):
    meshes, pts = small_batch(20, 13, levels=(2, 5), points=(2_000, 60_000))
    b = gsq.Batch(meshes, pts)
    d0 = b.run()
    o = b.tune()
    assert o["block_size"] in (64, 128) and o["queue_depth"] in (1, 4, 16) and o["leaf_size"] == 1
    depth = max(host_max_depth(v, f) for v, f in meshes)
    assert b.max_depth() == depth
    assert o["stack_depth"] in ((32, 64) if depth <= 31 else (64,))
    d1 = b.run()
    assert_bits_equal(d1, d0, "tuned run")


def test_batch_short_stack_falls_back(gsq):
    """A stack of 32 on trees deeper than 31 overflows; the run repeats with
    64 and returns exact results."""
    meshes, pts = small_batch(6, 17, levels=(6, 6), points=(2_000, 4_000))
    depth = max(host_max_depth(v, f) for v, f in meshes)
    b = gsq.Batch(meshes, pts)
    b.set_opts(stack_depth=32)
    d = b.run()
    check(b, d, None, [(e[0], None) for e in standalone(meshes, pts, closest=False)])
    assert b.opts()["stack_depth"] == (64 if depth > 31 else 32)


@pytest.mark.parametrize("opts", [dict(block_size=32, queue_depth=1, morton_bits=5),
                                  dict(block_size=96, queue_depth=16, morton_bits=23)])
def test_batch_options_do_not_change_results(gsq, opts):
    meshes, pts = small_batch(9, 29)
    b = gsq.Batch(meshes, pts)
    d0 = b.run()
    b.set_opts(**opts)
    assert_bits_equal(b.run(), d0, f"opts {opts}")


def test_batch_sample_against_oracle(gsq, port):
    """One mesh of a batch against the CPU oracle directly."""
    meshes, pts = small_batch(5, 37)
    b = gsq.Batch(meshes, pts, closest_points=True)
    d, cp = b.run(closest=True)
    k = 2
    v, f = meshes[k]
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    dref, cpref, _ = port.sdf_eval(h, pts[k], True, False, threads=8)
    assert_bits_equal(b.split(d)[k], dref, "distance vs oracle")
    assert_bits_equal(b.split(cp)[k], cpref, "closest point vs oracle")
