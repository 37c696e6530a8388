"""GPU: the local closest-point query of quest::DistributedClosestPoint.

Both forms (FP64 and FP32-certified nodes) must equal the reference's outputs
(golden fixture) and the oracle (live, larger clouds) bit for bit: index,
domain, position and distance, NaN patterns included.  Tolerance: bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import axom_gb300
from conftest import assert_bits_equal, golden

pytestmark = pytest.mark.gpu

PRECISIONS = [axom_gb300.PRECISION_FP64, axom_gb300.PRECISION_MIXED]


def check(got, want):
    for x, y, what in zip(got, want, ("index", "domain", "position", "distance")):
        assert_bits_equal(np.asarray(x), np.asarray(y), what)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("tag", ["all", "thr"])
def test_closest_point_matches_golden(gsq, precision, tag):
    g = golden("cp_points3000")
    cp = gsq.ClosestPoint(g["points"], g["domains"])
    if tag == "thr":
        cp.set_distance_threshold(0.05)
    got = cp.compute_closest_points(g["queries"], precision=precision)
    check(got, tuple(g[f"{tag}_{k}"] for k in ("idx", "dom", "pos", "dist")))


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("n", [0, 1, 2, 200_000])
def test_closest_point_matches_oracle(gsq, port, precision, n):
    r = np.random.default_rng(50 + n)
    pts = r.uniform(-5, 5, (n, 3))
    if n > 2:
        pts[n // 3:n // 3 + 1000] = pts[:1000]  # duplicates: ties
    dom = r.integers(0, 17, n).astype(np.int32)
    q = r.uniform(-6, 6, (100_000, 3))
    if n:
        q[:500] = pts[:min(n, 500)].repeat(500 // min(n, 500) + 1, 0)[:500]
    cp = gsq.ClosestPoint(pts, dom)
    h = port.cp(pts, dom)
    for t in (None, 0.2):
        thr = float(np.finfo(np.float64).max) if t is None else t * t
        if t is not None:
            cp.set_distance_threshold(t)
        check(cp.compute_closest_points(q, precision=precision), port.cp_query(h, q, thr, threads=8))


def test_closest_point_device_arrays(gsq, port):
    import torch
    r = np.random.default_rng(7)
    pts = r.normal(size=(50_000, 3))
    q = r.normal(size=(20_000, 3)) * 1.5
    cp = gsq.ClosestPoint(torch.from_numpy(pts).cuda())
    idx, dom, pos, dist = cp.compute_closest_points(torch.from_numpy(q).cuda())
    want = port.cp_query(port.cp(pts), q, threads=8)
    check((idx.cpu().numpy(), dom.cpu().numpy(), pos.cpu().numpy(), dist.cpu().numpy()), want)
