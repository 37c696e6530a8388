"""Oracles for the spatial-query hot path (TEST INFRASTRUCTURE ONLY).

Two CPU implementations live here, both used only as checkers (tests/,
``__graft_entry__.smoke``) or as the timed CPU baseline (``bench.py``):

* ``Port``  -- ``oracle/gsq_oracle.cpp``, a C++ restatement of axom's
  ``spin::BVH`` / ``quest::SignedDistance`` SEQ path, compiled here and on the
  GPU host with ``build_port()``.
* ``Ref``   -- ``oracle/_ref/libaxom_ref.so``, the reference's own code built
  from its sources by ``oracle/build_ref.py`` (only where the reference tree
  is present).

Both expose the same methods, so a test can run one check against either.
Arrays are numpy; boxes are (n, 6) float64 rows ``[xmin, ymin, zmin, xmax,
ymax, zmax]``; points (n, 3) float64 rows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SRC = HERE / "gsq_oracle.cpp"
PORT_LIB = HERE / "_build" / "libgsq_oracle.so"
REF_LIB = HERE / "_ref" / "libaxom_ref.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_uint32)


def build_port(force: bool = False) -> Path:
    """Compile the C++ restatement (no FMA contraction, OpenMP for threads)."""
    if PORT_LIB.exists() and not force and PORT_LIB.stat().st_mtime > PORT_SRC.stat().st_mtime:
        return PORT_LIB
    PORT_LIB.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           str(PORT_SRC), "-o", str(PORT_LIB)]
    subprocess.run(cmd, check=True)
    return PORT_LIB


def build_reference(reference: Path | None = None) -> Path | None:
    """Build the reference's own SEQ path when its sources are present
    (``reference`` defaults to the recipe's ``DEFAULT_REFERENCE``)."""
    import importlib
    br = importlib.import_module(__name__ + ".build_ref")
    reference = Path(reference) if reference is not None else br.DEFAULT_REFERENCE
    if not (reference / "src/axom/spin/BVH.hpp").exists():
        return None
    return br.build(reference, os.cpu_count() or 4)


def ref_available() -> bool:
    return REF_LIB.exists()


def _arr(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    if a is None:
        return None
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.uint32:
        return a.ctypes.data_as(_up)
    return a.ctypes.data_as(_ip)


class _Lib:
    prefix = ""

    def __init__(self, path: Path):
        self.lib = C.CDLL(str(path))
        p = self.prefix
        L = self.lib
        getattr(L, f"{p}bvh_create").restype = C.c_void_p
        getattr(L, f"{p}bvh_create").argtypes = [_dp, C.c_int, C.c_double]
        getattr(L, f"{p}bvh_destroy").argtypes = [C.c_void_p]
        getattr(L, f"{p}bvh_bounds").argtypes = [C.c_void_p, _dp]
        for f in ("bvh_find_boxes", "bvh_find_points"):
            getattr(L, p + f).restype = C.c_longlong
            getattr(L, p + f).argtypes = [C.c_void_p, _dp, C.c_int, _ip, _ip, C.POINTER(_ip)]
        getattr(L, f"{p}bvh_internals").restype = C.c_int
        getattr(L, f"{p}bvh_internals").argtypes = [_dp, C.c_int, C.c_double, _up, _ip, _ip, _ip, _ip, _dp, _dp, _dp]
        getattr(L, f"{p}sdf_create").restype = C.c_void_p
        getattr(L, f"{p}sdf_destroy").argtypes = [C.c_void_p]
        getattr(L, f"{p}sdf_eval").argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp, _dp, C.c_int]
        getattr(L, f"{p}sdf_counts").argtypes = [C.c_void_p, _dp, C.c_int, _ip, _ip, C.c_int]
        getattr(L, f"{p}sdf_mesh_bounds").argtypes = [C.c_void_p, _dp]
        getattr(L, f"{p}free").argtypes = [C.c_void_p]
        self.f = lambda name: getattr(L, p + name)

    # ---- BVH ----------------------------------------------------------
    def bvh(self, boxes, scale=1.000123):
        boxes = _arr(boxes, np.float64).reshape(-1, 6)
        return _Handle(self, self.f("bvh_create")(_p(boxes), boxes.shape[0], scale), "bvh_destroy")

    def bounds(self, h):
        out = np.empty(6)
        self.f("bvh_bounds")(h.ptr, _p(out))
        return out

    def _csr(self, fn, h, q, m, *extra):
        off = np.empty(m, np.int32)
        cnt = np.empty(m, np.int32)
        cp = _ip()
        total = fn(h.ptr, *extra, _p(off), _p(cnt), C.byref(cp))
        cand = np.ctypeslib.as_array(cp, shape=(max(total, 1),))[:total].copy() if total else np.empty(0, np.int32)
        self.f("free")(cp)
        return off, cnt, cand

    def find_boxes(self, h, q):
        q = _arr(q, np.float64).reshape(-1, 6)
        return self._csr(self.f("bvh_find_boxes"), h, q, q.shape[0], _p(q), q.shape[0])

    def find_points(self, h, p):
        p = _arr(p, np.float64).reshape(-1, 3)
        return self._csr(self.f("bvh_find_points"), h, p, p.shape[0], _p(p), p.shape[0])

    def find_boxes_counts(self, h, q):
        """Box-predicate calls of findBoundingBoxes' traversal, per query."""
        q = _arr(q, np.float64).reshape(-1, 6)
        nb = np.empty(q.shape[0], np.int32)
        fn = self.f("bvh_find_boxes_counts")
        fn.argtypes = [C.c_void_p, _dp, C.c_int, _ip]
        fn(h.ptr, _p(q), q.shape[0], _p(nb))
        return nb

    # ---- closest object point (DistributedClosestPoint's local query) -----
    def cp(self, pts, domains=None):
        p = _arr(pts, np.float64).reshape(-1, 3)
        d = _arr(domains, np.int32) if domains is not None else None
        fn = self.f("cp_create")
        fn.restype, fn.argtypes = C.c_void_p, [_dp, C.c_int, _ip]
        self.f("cp_destroy").argtypes = [C.c_void_p]
        return _Handle(self, fn(_p(p), p.shape[0], _p(d)), "cp_destroy")

    def cp_query(self, h, q, sq_threshold=float(np.finfo(np.float64).max), threads=1):
        """(index, domain, position (m,3), distance) per query point."""
        q = _arr(q, np.float64).reshape(-1, 3)
        m = q.shape[0]
        idx, dom = np.empty(m, np.int32), np.empty(m, np.int32)
        pos, dist = np.empty((m, 3)), np.empty(m)
        fn = self.f("cp_query")
        fn.argtypes = [C.c_void_p, _dp, C.c_int, C.c_double, _ip, _ip, _dp, _dp, C.c_int]
        fn(h.ptr, _p(q), m, sq_threshold, _p(idx), _p(dom), _p(pos), _p(dist), threads)
        return idx, dom, pos, dist

    def internals(self, boxes, scale=1.000123):
        boxes = _arr(boxes, np.float64).reshape(-1, 6)
        n = boxes.shape[0]
        out = dict(codes=np.empty(n, np.uint32), perm=np.empty(n, np.int32),
                   lchild=np.empty(n - 1, np.int32), rchild=np.empty(n - 1, np.int32),
                   parents=np.empty(2 * n - 1, np.int32), inner=np.empty((n - 1, 6)),
                   leaf=np.empty((n, 6)), bounds=np.empty(6))
        rc = self.f("bvh_internals")(_p(boxes), n, scale, *[_p(out[k]) for k in
                                     ("codes", "perm", "lchild", "rchild", "parents", "inner", "leaf", "bounds")])
        if rc != 0:
            raise ValueError("internals need n >= 2")
        return out

    # ---- SignedDistance -------------------------------------------------
    def sdf_eval(self, h, q, want_cp=False, want_normals=False, threads=1):
        q = _arr(q, np.float64).reshape(-1, 3)
        m = q.shape[0]
        out = np.empty(m)
        cp = np.empty((m, 3)) if want_cp else None
        nr = np.empty((m, 3)) if want_normals else None
        self.f("sdf_eval")(h.ptr, _p(q), m, _p(out), _p(cp), _p(nr), threads)
        return out, cp, nr

    def sdf_counts(self, h, q, threads=1):
        q = _arr(q, np.float64).reshape(-1, 3)
        m = q.shape[0]
        nb = np.empty(m, np.int32)
        nl = np.empty(m, np.int32)
        self.f("sdf_counts")(h.ptr, _p(q), m, _p(nb), _p(nl), threads)
        return nb, nl

    def mesh_bounds(self, h):
        out = np.empty(6)
        self.f("sdf_mesh_bounds")(h.ptr, _p(out))
        return out


class _Handle:
    def __init__(self, lib, ptr, dtor):
        self.lib, self.ptr, self.dtor = lib, C.c_void_p(ptr), dtor

    def __del__(self):
        try:
            if self.ptr:
                self.lib.f(self.dtor)(self.ptr)
                self.ptr = None
        except Exception:
            pass


class Port(_Lib):
    """The C++ restatement (always available once ``build_port`` ran)."""
    prefix = "orc_"

    def __init__(self, path: Path | None = None):
        super().__init__(path or build_port())
        L = self.lib
        L.orc_sdf_create.argtypes = [_dp, _dp, _dp, C.c_int, _ip, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_bvh_find_rays.restype = C.c_longlong
        L.orc_bvh_find_rays.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double, _ip, _ip, C.POINTER(_ip)]
        L.orc_ray_normalize.argtypes = [_dp, C.c_int, _dp]
        L.orc_bvh_layout.argtypes = [C.c_void_p, _dp, _ip, _ip]
        L.orc_bvh_size.restype = C.c_int
        L.orc_bvh_size.argtypes = [C.c_void_p]
        L.orc_sdf_tree.restype = C.c_void_p
        L.orc_sdf_tree.argtypes = [C.c_void_p]

    def sdf(self, x, y, z, cells, watertight=True, compute_sign=True):
        x, y, z = (_arr(a, np.float64) for a in (x, y, z))
        cells = _arr(cells, np.int32)
        npc = cells.shape[1] if cells.ndim == 2 else 3
        h = self.lib.orc_sdf_create(_p(x), _p(y), _p(z), x.size, _p(cells), cells.size // npc, npc,
                                    int(watertight), int(compute_sign))
        return _Handle(self, h, "sdf_destroy")

    def find_boxes_mt(self, h, q, threads):
        """findBoundingBoxes over contiguous sub-ranges of the queries on
        `threads` threads; the same CSR as find_boxes."""
        q = _arr(q, np.float64).reshape(-1, 6)
        fn = self.lib.orc_bvh_find_boxes_mt
        fn.restype = C.c_longlong
        fn.argtypes = [C.c_void_p, _dp, C.c_int, _ip, _ip, C.POINTER(_ip), C.c_int]
        m = q.shape[0]
        off = np.empty(m, np.int32)
        cnt = np.empty(m, np.int32)
        cp = _ip()
        total = fn(h.ptr, _p(q), m, _p(off), _p(cnt), C.byref(cp), threads)
        cand = np.ctypeslib.as_array(cp, shape=(max(total, 1),))[:total].copy() if total else np.empty(0, np.int32)
        self.f("free")(cp)
        return off, cnt, cand

    def normalize_rays(self, d):
        d = _arr(d, np.float64).reshape(-1, 3)
        out = np.empty_like(d)
        self.lib.orc_ray_normalize(_p(d), d.shape[0], _p(out))
        return out

    def find_rays(self, h, o, d_unit, tol=np.finfo(np.float64).eps):
        o = _arr(o, np.float64).reshape(-1, 3)
        d = _arr(d_unit, np.float64).reshape(-1, 3)
        m = o.shape[0]
        return self._csr(self.lib.orc_bvh_find_rays, h, o, m, _p(o), _p(d), m, tol)

    def layout(self, h):
        n = self.lib.orc_bvh_size(h.ptr)
        nodes = np.empty((2 * (n - 1), 6))
        ch = np.empty(2 * (n - 1), np.int32)
        leaf = np.empty(n, np.int32)
        self.lib.orc_bvh_layout(h.ptr, _p(nodes), _p(ch), _p(leaf))
        return nodes, ch, leaf


class Ref(_Lib):
    """The reference's own SEQ code (present only where it was built)."""
    prefix = "ref_"

    def __init__(self, path: Path = REF_LIB):
        if not Path(path).exists():
            raise FileNotFoundError(path)
        super().__init__(path)
        L = self.lib
        L.ref_sdf_create.argtypes = [_dp, _dp, _dp, C.c_int, _ip, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ref_bvh_find_rays.restype = C.c_longlong
        L.ref_bvh_find_rays.argtypes = [C.c_void_p, _dp, _dp, C.c_int, _ip, _ip, C.POINTER(_ip), _dp]

    def sdf(self, x, y, z, cells, watertight=True, compute_sign=True):
        x, y, z = (_arr(a, np.float64) for a in (x, y, z))
        cells = _arr(cells, np.int32)
        npc = cells.shape[1] if cells.ndim == 2 else 3
        h = self.lib.ref_sdf_create(_p(x), _p(y), _p(z), x.size, _p(cells), cells.size // npc, npc,
                                    int(watertight), int(compute_sign))
        return _Handle(self, h, "sdf_destroy")

    def stl_read(self, path):
        """quest::STLReader::read + getMesh: (nodes (n, 3), triangles (n/3, 3)), or None if read() failed."""
        fn = self.lib.ref_stl_read
        fn.restype, fn.argtypes = C.c_int, [C.c_char_p, C.POINTER(_dp), _ip, C.POINTER(_ip)]
        xyz, conn, nn = _dp(), _ip(), C.c_int()
        nc = fn(str(path).encode(), C.byref(xyz), C.byref(nn), C.byref(conn))
        if nc < 0:
            return None
        v = np.ctypeslib.as_array(xyz, shape=(max(nn.value, 1) * 3,))[: 3 * nn.value].reshape(-1, 3).copy()
        f = np.ctypeslib.as_array(conn, shape=(max(nc, 1) * 3,))[: 3 * nc].reshape(-1, 3).copy()
        self.lib.ref_free(xyz)
        self.lib.ref_free(conn)
        return v, f

    def find_rays(self, h, o, d_raw):
        """Rays built by primal::Ray(o, d): returns (off, cnt, cand, stored unit dirs)."""
        o = _arr(o, np.float64).reshape(-1, 3)
        d = _arr(d_raw, np.float64).reshape(-1, 3)
        m = o.shape[0]
        dirs = np.empty_like(d)
        off = np.empty(m, np.int32)
        cnt = np.empty(m, np.int32)
        cp = _ip()
        total = self.lib.ref_bvh_find_rays(h.ptr, _p(o), _p(d), m, _p(off), _p(cnt), C.byref(cp), _p(dirs))
        cand = np.ctypeslib.as_array(cp, shape=(max(total, 1),))[:total].copy() if total else np.empty(0, np.int32)
        self.lib.ref_free(cp)
        return off, cnt, cand, dirs
