"""Seeded synthetic workloads for the spatial-query path.

No public dataset or benchmark suite is involved; every input is generated
here from an explicit seed with ``numpy.random.Generator(PCG64(seed))``:

* ``random_boxes``   -- axis-aligned boxes, centres U[0,1]^3, per-axis side
  log-uniform in [1e-3, 1e-2] (the 100,000-box BVH workload).
* ``icosphere``      -- the 12-vertex icosahedron split ``level`` times at edge
  midpoints and projected to the unit sphere (20*4^L triangles, 10*4^L+2
  vertices), outward (counter-clockwise) winding.
* ``displace``       -- radial displacement r = 1 + 0.1 * sum_k sin(m_k theta +
  a_k) cos(n_k phi + b_k) over 8 random-phase terms with integer frequencies in
  1..6; theta = atan2(y, x), phi = acos(z).  r >= 0.2, so the surface stays
  closed, star-shaped and free of self-intersections.
* ``uniform_queries`` -- points uniform in the mesh box expanded by 20%.
* ``near_surface_queries`` -- points at a uniformly random (area-weighted)
  triangle, uniform barycentric position, offset along the face normal by
  +-10^U[-9,-3].
* ``uv_sphere`` / ``uniform_grid`` -- the UV-sphere surface and node grid used
  by axom's signed-distance unit test (quest/tests/quest_test_utilities.hpp:51,
  quest/tests/quest_signed_distance.cpp:66-81), restated.
"""
from __future__ import annotations

import math

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def random_boxes(n: int, seed: int) -> np.ndarray:
    g = rng(seed)
    c = g.uniform(0.0, 1.0, size=(n, 3))
    side = np.exp(g.uniform(math.log(1e-3), math.log(1e-2), size=(n, 3)))
    return np.concatenate([c - 0.5 * side, c + 0.5 * side], axis=1)


def icosphere(level: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: (vertices (V,3) float64, triangles (T,3) int32)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        key = np.minimum(e[:, 0], e[:, 1]) * nv + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = nv + inv.reshape(3, -1)  # midpoints of edges 01, 12, 20 per face
        m01, m12, m20 = m[0], m[1], m[2]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1),
            np.stack([m01, m12, m20], 1)], axis=0)
        v = np.concatenate([v, mid], axis=0)
    return v, f.astype(np.int32)


def quad_sphere(n: int) -> tuple[np.ndarray, np.ndarray]:
    """Cube with n x n quads per face projected to the unit sphere: (V,3), (6n^2, 4).

    Quads are wound counter-clockwise seen from outside."""
    e = np.eye(3)
    faces = [(np.array([1., -1, -1]), 2 * e[1], 2 * e[2]), (np.array([-1., -1, -1]), 2 * e[2], 2 * e[1]),
             (np.array([-1., 1, -1]), 2 * e[2], 2 * e[0]), (np.array([-1., -1, -1]), 2 * e[0], 2 * e[2]),
             (np.array([-1., -1, 1]), 2 * e[0], 2 * e[1]), (np.array([-1., -1, -1]), 2 * e[1], 2 * e[0])]
    t = np.arange(n + 1) / n
    pts, quads = [], []
    for k, (o, u, w) in enumerate(faces):
        I, J = np.meshgrid(t, t, indexing="ij")
        pts.append(o + I[..., None] * u + J[..., None] * w)
        base = k * (n + 1) ** 2
        i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
        idx = lambda a, b: base + a * (n + 1) + b  # noqa: E731
        quads.append(np.stack([idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)], -1).reshape(-1, 4))
    p = np.concatenate([q.reshape(-1, 3) for q in pts])
    quads = np.concatenate(quads)
    key = np.round(p * 4 * n).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    v = p[first]
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v, inv.reshape(-1)[quads].astype(np.int32)


def displace(v: np.ndarray, seed: int, amp: float = 0.1, terms: int = 8) -> np.ndarray:
    g = rng(seed)
    mk = g.integers(1, 7, size=terms)
    nk = g.integers(1, 7, size=terms)
    ak = g.uniform(0, 2 * np.pi, size=terms)
    bk = g.uniform(0, 2 * np.pi, size=terms)
    theta = np.arctan2(v[:, 1], v[:, 0])
    phi = np.arccos(np.clip(v[:, 2], -1.0, 1.0))
    r = 1.0 + amp * np.sum(np.sin(np.outer(theta, mk) + ak) * np.cos(np.outer(phi, nk) + bk), axis=1)
    return v * r[:, None]


def displaced_icosphere(level: int, seed: int = 1234) -> tuple[np.ndarray, np.ndarray]:
    v, f = icosphere(level)
    return displace(v, seed), f


def sliver_sheet(seed: int, n: int = 40) -> tuple[np.ndarray, np.ndarray]:
    """An open jittered grid surface with many slivers; every 17th triangle is
    collapsed onto a line (zero area)."""
    g = rng(seed)
    x, y = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij")
    z = 0.05 * np.sin(6 * x) * np.cos(5 * y)
    v = np.stack([x, y, z], -1).reshape(-1, 3)
    v[:, :2] += g.normal(scale=0.004, size=(v.shape[0], 2))
    i, j = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="ij")
    a = (i * n + j).ravel()
    f = np.concatenate([np.stack([a, a + n, a + n + 1], 1), np.stack([a, a + n + 1, a + 1], 1)]).astype(np.int32)
    deg = f[::17]
    v[deg[:, 2]] = 0.5 * (v[deg[:, 0]] + v[deg[:, 1]])
    return v, f


def expanded_box(v: np.ndarray, factor: float = 1.2) -> tuple[np.ndarray, np.ndarray]:
    lo, hi = v.min(axis=0), v.max(axis=0)
    c, h = 0.5 * (lo + hi), 0.5 * (hi - lo) * factor
    return c - h, c + h


def uniform_queries(v: np.ndarray, m: int, seed: int, factor: float = 1.2) -> np.ndarray:
    lo, hi = expanded_box(v, factor)
    return rng(seed).uniform(lo, hi, size=(m, 3))


def near_surface_queries(v: np.ndarray, f: np.ndarray, m: int, seed: int) -> np.ndarray:
    g = rng(seed)
    a, b, c = v[f[:, 0]], v[f[:, 1]], v[f[:, 2]]
    n = np.cross(b - a, c - a)
    area = np.linalg.norm(n, axis=1)
    tri = g.choice(f.shape[0], size=m, p=area / area.sum())
    r1, r2 = g.uniform(size=m), g.uniform(size=m)
    s = np.sqrt(r1)
    w0, w1, w2 = 1 - s, s * (1 - r2), s * r2
    p = w0[:, None] * a[tri] + w1[:, None] * b[tri] + w2[:, None] * c[tri]
    nu = n[tri] / area[tri, None]
    off = 10.0 ** g.uniform(-9, -3, size=m) * np.where(g.uniform(size=m) < 0.5, -1.0, 1.0)
    return p + off[:, None] * nu


def mixed_queries(v: np.ndarray, f: np.ndarray, m: int, seed: int) -> np.ndarray:
    """Half uniform in the 1.2x box, half near the surface, interleaved."""
    h = m // 2
    u = uniform_queries(v, m - h, seed)
    s = near_surface_queries(v, f, h, seed + 1000)
    out = np.empty((m, 3))
    out[0::2][: m - h] = u
    out[1::2][:h] = s
    return out


def random_rotation(r: np.random.Generator) -> np.ndarray:
    """A uniformly random rotation matrix (QR of a Gaussian matrix, sign-fixed)."""
    q, rr = np.linalg.qr(r.normal(size=(3, 3)))
    q *= np.sign(np.diag(rr))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def batch_meshes(n: int, seed: int, levels=(2, 6), points=(1_000, 1_000_000), point_scale: float = 1.0):
    """The batched workload: n icospheres, each at a uniformly random level in
    ``levels`` (320..81,920 triangles for 2..6), randomly rotated, scaled in
    [0.5, 2] and translated in [-10, 10]^3, each with a log-uniform number of
    points in ``points`` (times ``point_scale``) uniform in its bounding box
    expanded by 20%.  Returns (meshes [(V, F)], points [(M_k, 3)])."""
    r = rng(seed)
    cache = {}
    meshes, pts = [], []
    for k in range(n):
        level = int(r.integers(levels[0], levels[1] + 1))
        if level not in cache:
            cache[level] = icosphere(level)
        v0, f = cache[level]
        v = (v0 @ random_rotation(r).T) * r.uniform(0.5, 2.0) + r.uniform(-10.0, 10.0, size=3)
        lo, hi = np.log(points[0]), np.log(points[1])
        m = max(1, int(round(np.exp(r.uniform(lo, hi)) * point_scale)))
        meshes.append((v, f))
        pts.append(uniform_queries(v, m, seed * 7919 + k))
    return meshes, pts


def uv_sphere(center=(0.0, 0.0, 0.0), radius=0.5, theta_res=25, phi_res=25):
    """UV sphere (quest/tests/quest_test_utilities.hpp:51-150), restated."""
    deg = math.pi / 180.0
    pts = [(center[0], center[1], center[2] + radius), (center[0], center[1], center[2] - radius)]
    dphi = (180 * deg) / float(phi_res - 1)
    dtheta = (360 * deg) / float(theta_res - 1)
    for i in range(theta_res):
        th = i * dtheta
        for j in range(phi_res - 2):
            ph = j * dphi
            rr = radius * math.sin(ph)
            pts.append((rr * math.cos(th) + center[0], rr * math.sin(th) + center[1],
                        radius * math.cos(ph) + center[2]))
    pr = phi_res - 2
    stride = pr * theta_res
    cells = []
    for i in range(theta_res):
        cells.append((0, (pr * (i + 1) % stride) + 2, pr * i + 2))
    off = phi_res - 1
    for i in range(theta_res):
        cells.append((1, (pr * (i + 1) % stride) + off, pr * i + off))
    for i in range(theta_res):
        for j in range(phi_res - 3):
            c0 = pr * i + j + 2
            c2 = ((pr * (i + 1) + j) % stride) + 3
            cells.append((c0, c0 + 1, c2))
            cells.append((c0, c2, c2 - 1))
    return np.array(pts, dtype=np.float64), np.array(cells, dtype=np.int32)


def uniform_grid(lo, hi, n: int) -> np.ndarray:
    """Nodes of an n^3 uniform mesh (mint::UniformMesh node order, i fastest)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    h = (hi - lo) / (n - 1)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return np.stack([lo[0] + i.ravel() * h[0], lo[1] + j.ravel() * h[1], lo[2] + k.ravel() * h[2]], axis=1)


def uniform_cells(lo, hi, n: int) -> np.ndarray:
    """Cell boxes of an n^3-node uniform mesh (cells i fastest), (c,6)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    h = (hi - lo) / (n - 1)
    k, j, i = np.meshgrid(np.arange(n - 1), np.arange(n - 1), np.arange(n - 1), indexing="ij")
    idx = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    return np.concatenate([lo + idx * h, lo + (idx + 1) * h], axis=1)
