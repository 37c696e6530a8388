"""GPU: the mixed-precision form (FP32 certified traversal, FP64 refine).

Its distances and closest points must equal the FP64 form (and so the
reference) bit for bit, with identical signs; the audit mode re-evaluates every
triangle the FP32 certificate skipped in FP64 and must find no contradiction.
Tolerances: distances and closest points bit-exact (the stated bar of 1e-12
relative is met with margin); unit normals 1e-12 absolute."""
from __future__ import annotations

import numpy as np
import pytest

import axom_gb300
from axom_gb300 import workloads as W
from conftest import assert_bits_equal, golden

pytestmark = pytest.mark.gpu

FIXTURES = ["sdf_uvsphere", "sdf_ico3", "sdf_ico3_open", "sdf_ico3_unsigned", "sdf_quad12"]


@pytest.mark.parametrize("name", FIXTURES)
def test_mixed_matches_golden(gsq, name):
    g = golden(name)
    sd = gsq.SignedDistance(g["vertices"], g["cells"], bool(g["watertight"]), bool(g["sign"]),
                            precision=axom_gb300.PRECISION_MIXED)
    d, cp, nr = sd.compute_distances(g["queries"], closest=True, normals=True)
    assert_bits_equal(d, g["dist"], "distance")
    assert_bits_equal(cp, g["closest"], "closest point")
    np.testing.assert_allclose(nr, g["normals"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", ["ico5", "ico6", "quad30", "slivers", "open_ico5"])
def test_mixed_equals_fp64_with_audit(gsq, case):
    watertight = True
    if case.startswith("ico"):
        v, f = W.displaced_icosphere(int(case[3]), 7)
    elif case == "quad30":
        v, f = W.quad_sphere(30)
        v = W.displace(v, 8)
    elif case == "slivers":
        v, f = W.sliver_sheet(3)
        watertight = False
    else:
        v, f = W.displaced_icosphere(5, 9)
        f = f[np.arange(f.shape[0]) % 5 != 0]
        watertight = False
    tri = f[:, :3]
    q = np.concatenate([W.uniform_queries(v, 30000, 1), W.near_surface_queries(v, tri, 30000, 2),
                        v[np.arange(0, v.shape[0], 7)]])  # exactly on vertices too
    sd = gsq.SignedDistance(v, f, is_watertight=watertight, precision=axom_gb300.PRECISION_FP64)
    d64, cp64, n64 = sd.compute_distances(q, closest=True, normals=True)
    sd.set_precision(axom_gb300.PRECISION_MIXED)
    sd.set_audit(True)
    dm, cpm, nm = sd.compute_distances(q, closest=True, normals=True)
    st = sd.mixed_stats()
    assert st["violations"] == 0, st
    assert_bits_equal(dm, d64, "distance")
    assert_bits_equal(cpm, cp64, "closest point")
    np.testing.assert_allclose(nm, n64, rtol=0, atol=1e-12)
    assert st["leaf_skipped"] > 0
    # without normals the sign is certified in FP32 where it can be; the audit
    # checks every certified sign against the FP64 pseudo-normal test
    dm2 = sd.compute_distances(q)
    assert sd.mixed_stats()["violations"] == 0
    assert_bits_equal(dm2, d64, "distance, FP32-certified signs (audited)")
    sd.set_audit(False)
    assert_bits_equal(sd.compute_distances(q), d64, "distance without audit")


def test_mixed_audit_fine_mesh(gsq):
    """Level-8 triangles are small (edges ~0.008), where the reference's fixed
    fuzzy EPS moves its closest point the most; the audit checks every skip
    and every queued candidate's distance bounds."""
    import torch
    v, f = W.displaced_icosphere(8, 1234)
    q = torch.from_numpy(W.mixed_queries(v, f, 1 << 20, 9)).cuda()
    sd = gsq.SignedDistance(v, f, precision=axom_gb300.PRECISION_FP64)
    d64, cp64, _ = sd.compute_distances(q, closest=True)
    sd.set_precision(axom_gb300.PRECISION_MIXED)
    sd.set_audit(True)
    dm, cpm, _ = sd.compute_distances(q, closest=True)
    st = sd.mixed_stats()
    assert st["violations"] == 0, st
    assert torch.equal(dm.view(torch.int64), d64.view(torch.int64))
    assert torch.equal(cpm.view(torch.int64), cp64.view(torch.int64))


def test_mixed_full_size_near_surface(gsq, port):
    """Level-8 mesh (1,310,720 triangles), 16M points: half uniform, half at
    offsets 1e-9..1e-3 along the normal.  Mixed vs FP64 on the GPU over every
    point: zero sign mismatches and zero relative error; and a 40,000-point
    stratified sample (half of it near the surface) against the oracle, bit
    for bit."""
    import torch
    v, f = W.displaced_icosphere(8, 1234)
    m = 1 << 24
    q_host = W.mixed_queries(v, f, m, 4)
    q = torch.from_numpy(q_host).cuda()
    sd = gsq.SignedDistance(v, f, precision=axom_gb300.PRECISION_FP64)
    d64 = sd.compute_distances(q)
    sd.set_precision(axom_gb300.PRECISION_MIXED)
    dm = sd.compute_distances(q)
    assert int((torch.sign(dm) != torch.sign(d64)).sum()) == 0
    rel = ((dm - d64).abs() / d64.abs().clamp_min(1e-300)).max().item()
    assert rel <= 1e-12
    assert torch.equal(dm.view(torch.int64), d64.view(torch.int64))
    idx = np.linspace(0, m - 2, 20000).astype(np.int64) // 2 * 2
    idx = np.concatenate([idx, idx + 1])  # even: uniform, odd: near the surface
    h = port.sdf(v[:, 0], v[:, 1], v[:, 2], f)
    pd, _, _ = port.sdf_eval(h, q_host[idx], threads=16)
    assert_bits_equal(dm[torch.from_numpy(idx).cuda()].cpu().numpy(), pd, "oracle sample")
