"""axom_gb300: GB300-native spatial queries (axom spin::BVH + quest::SignedDistance).

Python mirror of the reference interface over the C ABI in ``include/gsq.h``
(``libgsq.so``, built by ``axom_gb300.build``).  Class and method names follow
the reference:

* ``BVH``            -- ``spin::BVH<3, Exec, double>`` (spin/BVH.hpp:129-568):
  ``initialize``, ``find_points``, ``find_rays``, ``find_bounding_boxes``,
  ``get_bounds``, ``set/get_scale_factor``, ``set/get_tolerance``.
* ``SignedDistance`` -- ``quest::SignedDistance<3, Exec>``
  (quest/SignedDistance.hpp:147-605): ``compute_distance``,
  ``compute_distances``, ``get_mesh_bounds``, ``get_bvh_tree``.
* ``ClosestPoint``   -- the local query of ``quest::DistributedClosestPoint``
  (quest/detail/DistributedClosestPointImpl.hpp:883-901, 1002-1050):
  ``set_distance_threshold``, ``compute_closest_points``.
* ``Batch``          -- many meshes and point sets in one CUDA graph (no
  reference counterpart).

Arrays may be numpy arrays (host memory) or torch tensors (host or CUDA); the
C ABI classifies each pointer.  Outputs are numpy arrays for host inputs and
torch CUDA tensors for device inputs.  There is no CPU fallback: without the
compiled library or a CUDA device every call raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

__all__ = ["GsqError", "BVH", "SignedDistance", "ClosestPoint", "Batch", "load", "PRECISION_FP64",
           "PRECISION_MIXED"]

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libgsq.so"

GSQ_OK = 0
BVH_BUILD_OK = 0
PRECISION_FP64 = 0
PRECISION_MIXED = 1
DEFAULT_SCALE_FACTOR = 1.000123
DEFAULT_TOLERANCE = float(np.finfo(np.float64).eps)

_lib = None
_vp, _dp, _ip, _up = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint32)
_i64p = C.POINTER(C.c_int64)


class GsqError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gsq error {code}: {msg}")
        self.code = code


class SdfOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("sort_queries", C.c_int32), ("block_size", C.c_int32),
                ("audit", C.c_int32), ("queue_depth", C.c_int32), ("reserved", C.c_int32 * 3)]


class BvhView(C.Structure):
    """gsq_bvh_view: device pointers for user kernels (include/gsq_device.cuh)."""
    _fields_ = [("nodes", C.c_void_p), ("leaf_ids", C.c_void_p), ("num_leaves", C.c_int32),
                ("reserved", C.c_int32)]


class BatchOpts(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("queue_depth", C.c_int32), ("stack_depth", C.c_int32),
                ("morton_bits", C.c_int32), ("leaf_size", C.c_int32), ("closest_points", C.c_int32),
                ("reserved", C.c_int32 * 2)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


# (name, restype, argtypes) of every entry point declared in include/gsq.h
SIGNATURES = [
    ("gsq_last_error", C.c_char_p, []),
    ("gsq_selftest_bounded_wait", C.c_int, [_vp]),
    ("gsq_version", C.c_char_p, []),
    ("gsq_kernel_launches", C.c_int64, []),
    ("gsq_free", C.c_int, [_vp]),
    ("gsq_memcpy", C.c_int, [_vp, _vp, C.c_size_t]),
    ("gsq_bvh_create", C.c_int, [C.POINTER(_vp)]),
    ("gsq_bvh_destroy", C.c_int, [_vp]),
    ("gsq_bvh_set_scale_factor", C.c_int, [_vp, C.c_double]),
    ("gsq_bvh_get_scale_factor", C.c_int, [_vp, _dp]),
    ("gsq_bvh_set_tolerance", C.c_int, [_vp, C.c_double]),
    ("gsq_bvh_get_tolerance", C.c_int, [_vp, _dp]),
    ("gsq_bvh_build", C.c_int, [_vp, _vp, C.c_int32, _vp]),
    ("gsq_bvh_bounds", C.c_int, [_vp, _dp, _dp]),
    ("gsq_bvh_num_leaves", C.c_int, [_vp, _ip]),
    ("gsq_bvh_find_boxes", C.c_int, [_vp, _vp, C.c_int32, _vp, _vp, C.POINTER(_vp), _i64p, _vp]),
    ("gsq_bvh_find_points", C.c_int, [_vp, _vp, C.c_int32, _vp, _vp, C.POINTER(_vp), _i64p, _vp]),
    ("gsq_bvh_find_rays", C.c_int, [_vp, _vp, _vp, C.c_int32, _vp, _vp, C.POINTER(_vp), _i64p, _vp]),
    ("gsq_ray_normalize", C.c_int, [_dp, C.c_int32, _dp]),
    ("gsq_bvh_export", C.c_int, [_vp, _dp, _ip, _ip, _up]),
    ("gsq_bvh_last_build_ms", C.c_int, [_vp, C.POINTER(C.c_float)]),
    ("gsq_bvh_last_find_ms", C.c_int, [_vp, C.POINTER(C.c_float)]),
    ("gsq_sdf_opts_init", C.c_int, [C.POINTER(SdfOpts)]),
    ("gsq_sdf_create", C.c_int, [C.POINTER(_vp), _vp, _vp, _vp, C.c_int32, _vp, C.c_int32, C.c_int32, C.c_int32,
                                 C.c_int32, C.POINTER(SdfOpts), _vp]),
    ("gsq_sdf_destroy", C.c_int, [_vp]),
    ("gsq_sdf_set_opts", C.c_int, [_vp, C.POINTER(SdfOpts)]),
    ("gsq_sdf_eval", C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp, _vp, _vp]),
    ("gsq_sdf_mesh_bounds", C.c_int, [_vp, _dp, _dp]),
    ("gsq_sdf_get_bvh", C.c_int, [_vp, C.POINTER(_vp)]),
    ("gsq_sdf_last_eval_ms", C.c_int, [_vp, C.POINTER(C.c_float)]),
    ("gsq_sdf_mixed_stats", C.c_int, [_vp, _i64p]),
    ("gsq_sdf_backward", C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp, _vp, _vp]),
    ("gsq_sdf_eval_tri", C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp, _vp]),
    ("gsq_sdf_backward_tri", C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("gsq_sdf_eval_noalloc", C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp, _vp]),
    ("gsq_stl_read", C.c_int, [C.c_char_p, C.POINTER(_dp), _ip, C.POINTER(_ip), _ip]),
    ("gsq_bvh_get_view", C.c_int, [_vp, C.POINTER(BvhView)]),
    ("gsq_cpq_create", C.c_int, [C.POINTER(_vp), _vp, C.c_int32, _vp, _vp]),
    ("gsq_cpq_destroy", C.c_int, [_vp]),
    ("gsq_cpq_query", C.c_int, [_vp, _vp, C.c_int32, C.c_double, C.c_int32, _vp, _vp, _vp, _vp, _vp]),
    ("gsq_cpq_last_ms", C.c_int, [_vp, C.POINTER(C.c_float)]),
    ("gsq_batch_opts_init", C.c_int, [_vp]),
    ("gsq_batch_create", C.c_int, [C.POINTER(_vp), C.c_int32, _vp, _vp, _vp, C.c_int32, _vp, C.c_int32, C.c_int32,
                                   _vp, _vp]),
    ("gsq_batch_destroy", C.c_int, [_vp]),
    ("gsq_batch_set_vertices", C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    ("gsq_batch_set_points", C.c_int, [_vp, _vp, _vp]),
    ("gsq_batch_run", C.c_int, [_vp, _vp, _vp, _vp]),
    ("gsq_batch_device_output", C.c_int, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
    ("gsq_batch_tune", C.c_int, [_vp, _vp]),
    ("gsq_batch_get_opts", C.c_int, [_vp, _vp]),
    ("gsq_batch_set_opts", C.c_int, [_vp, _vp]),
    ("gsq_batch_last_ms", C.c_int, [_vp, C.POINTER(C.c_float)]),
    ("gsq_batch_max_depth", C.c_int, [_vp, _ip]),
    # the quest C interface (include/gsq_quest.h)
    ("QUEST_signed_distance_init_serial", C.c_int, [C.c_char_p]),
    ("QUEST_signed_distance_init_serial_bufferify", C.c_int, [C.c_char_p, C.c_int]),
    ("QUEST_signed_distance_initialized", C.c_bool, []),
    ("QUEST_signed_distance_get_mesh_bounds", None, [_dp, _dp]),
    ("QUEST_signed_distance_set_dimension", None, [C.c_int]),
    ("QUEST_signed_distance_set_closed_surface", None, [C.c_bool]),
    ("QUEST_signed_distance_set_compute_signs", None, [C.c_bool]),
    ("QUEST_signed_distance_set_allocator", None, [C.c_int]),
    ("QUEST_signed_distance_set_verbose", None, [C.c_bool]),
    ("QUEST_signed_distance_use_shared_memory", None, [C.c_bool]),
    ("QUEST_signed_distance_set_execution_space", None, [C.c_int]),
    ("QUEST_signed_distance_evaluate_0", C.c_double, [C.c_double, C.c_double, C.c_double]),
    ("QUEST_signed_distance_evaluate_1", C.c_double, [C.c_double, C.c_double, C.c_double] + [_dp] * 6),
    ("QUEST_signed_distance_finalize", None, []),
    ("gsq_quest_init_mesh", C.c_int, [_vp, _vp, _vp, C.c_int32, _vp, C.c_int32]),
    ("gsq_quest_evaluate_points", None, [_vp, _vp, _vp, C.c_int32, _vp]),
    ("gsq_quest_set_precision", C.c_int, [C.c_int32]),
    ("gsq_quest_handle", C.c_int, [C.POINTER(_vp)]),
]
NOALLOC_MAX_QUERIES = 262144  # GSQ_NOALLOC_MAX_QUERIES in include/gsq.h


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads libgsq.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: run axom_gb300.build.build() (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    if path is None:
        _lib = lib
    return lib


def _check(rc: int):
    if rc != GSQ_OK:
        raise GsqError(rc, load().gsq_last_error().decode())


# ---- array plumbing -----------------------------------------------------------
def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _stream():
    try:
        import torch
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    except ImportError:
        pass
    return None


class _Arr:
    """A contiguous array view with a raw pointer (host numpy or torch)."""

    def __init__(self, a, dtype, cols=None):
        if _is_torch(a):
            import torch
            tdt = {np.float64: torch.float64, np.int32: torch.int32}[dtype]
            t = a.to(tdt).contiguous()
            if cols:
                t = t.reshape(-1, cols)
            self.obj, self.ptr, self.device = t, t.data_ptr(), t.is_cuda
            self.n = t.shape[0] if t.dim() else 1
            self.torch_device = t.device
        else:
            x = np.ascontiguousarray(a, dtype=dtype)
            if cols:
                x = x.reshape(-1, cols)
            self.obj, self.ptr, self.device = x, x.ctypes.data, False
            self.n = x.shape[0] if x.ndim else 1
            self.torch_device = None

    def empty(self, shape, dtype):
        if self.device:
            import torch
            tdt = {np.float64: torch.float64, np.int32: torch.int32}[dtype]
            return torch.empty(shape, dtype=tdt, device=self.torch_device)
        return np.empty(shape, dtype=dtype)


def _ptr(a):
    return a.data_ptr() if _is_torch(a) else a.ctypes.data


class BVH:
    """spin::BVH<3, CUDA_EXEC, double> on the GB300 (spin/BVH.hpp:129-568)."""

    def __init__(self, boxes=None, num_items: int | None = None, scale_factor: float = DEFAULT_SCALE_FACTOR,
                 tolerance: float = DEFAULT_TOLERANCE, _handle=None):
        self._lib = load()
        self._owned = _handle is None
        if _handle is None:
            h = _vp()
            _check(self._lib.gsq_bvh_create(C.byref(h)))
            self._h = h
            self.set_scale_factor(scale_factor)
            self.set_tolerance(tolerance)
        else:
            self._h = _handle
        if boxes is not None:
            self.initialize(boxes, num_items)

    def __del__(self):
        if getattr(self, "_owned", False) and getattr(self, "_h", None):
            self._lib.gsq_bvh_destroy(self._h)
            self._h = None

    def set_scale_factor(self, s: float):
        _check(self._lib.gsq_bvh_set_scale_factor(self._h, s))

    def get_scale_factor(self) -> float:
        v = C.c_double()
        _check(self._lib.gsq_bvh_get_scale_factor(self._h, C.byref(v)))
        return v.value

    def set_tolerance(self, t: float):
        _check(self._lib.gsq_bvh_set_tolerance(self._h, t))

    def get_tolerance(self) -> float:
        v = C.c_double()
        _check(self._lib.gsq_bvh_get_tolerance(self._h, C.byref(v)))
        return v.value

    def initialize(self, boxes, num_items: int | None = None) -> int:
        """Builds over (n, 6) boxes [xmin, ymin, zmin, xmax, ymax, zmax]."""
        b = _Arr(boxes, np.float64, 6)
        n = b.n if num_items is None else int(num_items)
        _check(self._lib.gsq_bvh_build(self._h, C.c_void_p(b.ptr), n, _stream()))
        return BVH_BUILD_OK

    def get_bounds(self):
        lo, hi = np.empty(3), np.empty(3)
        _check(self._lib.gsq_bvh_bounds(self._h, lo.ctypes.data_as(_dp), hi.ctypes.data_as(_dp)))
        return lo, hi

    def num_leaves(self) -> int:
        v = C.c_int32()
        _check(self._lib.gsq_bvh_num_leaves(self._h, C.byref(v)))
        return v.value

    def last_build_ms(self) -> float:
        v = C.c_float()
        _check(self._lib.gsq_bvh_last_build_ms(self._h, C.byref(v)))
        return v.value

    def last_find_ms(self) -> float:
        """Device time of the last find's traversal passes and scan."""
        v = C.c_float()
        _check(self._lib.gsq_bvh_last_find_ms(self._h, C.byref(v)))
        return v.value

    def get_view(self) -> BvhView:
        """BVH::getTraverser: device pointers for user kernels (include/gsq_device.cuh)."""
        v = BvhView()
        _check(self._lib.gsq_bvh_get_view(self._h, C.byref(v)))
        return v

    def _find(self, fn, arrs, m, like: _Arr):
        off = like.empty(m, np.int32)
        cnt = like.empty(m, np.int32)
        cand = _vp()
        total = C.c_int64()
        _check(fn(self._h, *[C.c_void_p(a.ptr) for a in arrs], m, C.c_void_p(_ptr(off)), C.c_void_p(_ptr(cnt)),
                  C.byref(cand), C.byref(total), _stream()))
        t = total.value
        try:
            if like.device:
                import torch
                out = torch.empty(t, dtype=torch.int32, device=like.torch_device)
                if t:
                    _check(self._lib.gsq_memcpy(C.c_void_p(out.data_ptr()), cand, C.c_size_t(4 * t)))
            else:
                out = np.ctypeslib.as_array(C.cast(cand, _ip), shape=(max(t, 1),))[:t].copy() if t else \
                    np.empty(0, np.int32)
        finally:
            self._lib.gsq_free(cand)
        return off, cnt, out

    def find_bounding_boxes(self, boxes):
        """(offsets, counts, candidates) for (m, 6) query boxes."""
        q = _Arr(boxes, np.float64, 6)
        return self._find(self._lib.gsq_bvh_find_boxes, [q], q.n, q)

    def find_points(self, points):
        q = _Arr(points, np.float64, 3)
        return self._find(self._lib.gsq_bvh_find_points, [q], q.n, q)

    def find_rays(self, origins, directions):
        """Rays with stored unit directions (see normalize_rays)."""
        o = _Arr(origins, np.float64, 3)
        d = _Arr(directions, np.float64, 3)
        return self._find(self._lib.gsq_bvh_find_rays, [o, d], o.n, o)

    def export(self):
        """Reference LinearBVH layout: (node_boxes, children, leaf_ids, codes)."""
        n = self.num_leaves()
        nodes = np.empty((2 * (n - 1), 6))
        ch = np.empty(2 * (n - 1), np.int32)
        leaf = np.empty(n, np.int32)
        codes = np.empty(n, np.uint32)
        _check(self._lib.gsq_bvh_export(self._h, nodes.ctypes.data_as(_dp), ch.ctypes.data_as(_ip),
                                        leaf.ctypes.data_as(_ip), codes.ctypes.data_as(_up)))
        return nodes, ch, leaf, codes


def read_stl(path) -> tuple[np.ndarray, np.ndarray]:
    """quest::STLReader (quest/readers/STLReader.cpp): (nodes (n, 3), triangles
    (n/3, 3)) of an ASCII or binary STL file, three nodes per triangle."""
    lib = load()
    xyz, cells = _dp(), _ip()
    nn, nc = C.c_int32(), C.c_int32()
    _check(lib.gsq_stl_read(str(path).encode(), C.byref(xyz), C.byref(nn), C.byref(cells), C.byref(nc)))
    try:
        v = np.ctypeslib.as_array(xyz, shape=(max(nn.value, 1) * 3,))[: 3 * nn.value].reshape(-1, 3).copy()
        f = np.ctypeslib.as_array(cells, shape=(max(nc.value, 1) * 3,))[: 3 * nc.value].reshape(-1, 3).copy()
    finally:
        lib.gsq_free(xyz)
        lib.gsq_free(cells)
    return v, f


def normalize_rays(directions) -> np.ndarray:
    """primal::Ray's direction normalisation (Vector::unitVector) on the host."""
    d = np.ascontiguousarray(directions, dtype=np.float64).reshape(-1, 3)
    out = np.empty_like(d)
    _check(load().gsq_ray_normalize(d.ctypes.data_as(_dp), d.shape[0], out.ctypes.data_as(_dp)))
    return out


class SignedDistance:
    """quest::SignedDistance<3, CUDA_EXEC> on the GB300 (quest/SignedDistance.hpp:147-605).

    ``vertices`` (V, 3) and ``cells`` (C, 3 or 4) describe an unstructured
    single-shape surface mesh (triangles or quads)."""

    def __init__(self, vertices, cells, is_watertight: bool = True, compute_sign: bool = True,
                 precision: int = PRECISION_FP64, sort_queries: bool = True):
        self._lib = load()
        v = np.ascontiguousarray(vertices, dtype=np.float64).reshape(-1, 3) if not _is_torch(vertices) \
            else vertices.detach().to("cpu").double().reshape(-1, 3).numpy()
        c = np.ascontiguousarray(cells, dtype=np.int32) if not _is_torch(cells) \
            else cells.detach().to("cpu").int().numpy()
        npc = c.shape[1] if c.ndim == 2 else 3
        self.num_vertices = v.shape[0]
        x, y, z = (np.ascontiguousarray(v[:, k]) for k in range(3))
        self._opts = SdfOpts()
        _check(self._lib.gsq_sdf_opts_init(C.byref(self._opts)))
        self._opts.precision = precision
        self._opts.sort_queries = int(sort_queries)
        h = _vp()
        _check(self._lib.gsq_sdf_create(C.byref(h), C.c_void_p(x.ctypes.data), C.c_void_p(y.ctypes.data),
                                        C.c_void_p(z.ctypes.data), v.shape[0], C.c_void_p(c.ctypes.data),
                                        c.size // npc, npc, int(is_watertight), int(compute_sign),
                                        C.byref(self._opts), _stream()))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gsq_sdf_destroy(self._h)
            self._h = None

    def set_precision(self, precision: int):
        self._opts.precision = precision
        _check(self._lib.gsq_sdf_set_opts(self._h, C.byref(self._opts)))

    def set_sort_queries(self, on: bool):
        self._opts.sort_queries = int(on)
        _check(self._lib.gsq_sdf_set_opts(self._h, C.byref(self._opts)))

    def set_audit(self, on: bool):
        self._opts.audit = int(on)
        _check(self._lib.gsq_sdf_set_opts(self._h, C.byref(self._opts)))

    def mixed_stats(self) -> dict:
        c = (C.c_int64 * 4)()
        _check(self._lib.gsq_sdf_mixed_stats(self._h, c))
        return {"violations": c[0], "node_fp64": c[1], "leaf_fp64": c[2], "leaf_skipped": c[3]}

    def compute_distances(self, points, closest: bool = False, normals: bool = False, out=None):
        """Signed distances of (m, 3) points; optional closest points and unit normals.

        ``out`` (optional) is a caller-owned (m,) float64 buffer, host or device."""
        p = _Arr(points, np.float64, 3)
        m = p.n
        out = p.empty(m, np.float64) if out is None else out
        cp = p.empty((m, 3), np.float64) if closest else None
        nr = p.empty((m, 3), np.float64) if normals else None
        base = p.ptr
        _check(self._lib.gsq_sdf_eval(self._h, C.c_void_p(base), C.c_void_p(base + 8), C.c_void_p(base + 16), 3, m,
                                      C.c_void_p(_ptr(out)), C.c_void_p(_ptr(cp)) if cp is not None else None,
                                      C.c_void_p(_ptr(nr)) if nr is not None else None, _stream()))
        if closest or normals:
            return out, cp, nr
        return out

    def compute_distances_soa(self, x, y, z, out):
        """signed_distance_evaluate(x, y, z, n, phi) form: three coordinate arrays."""
        xs, ys, zs = (_Arr(a, np.float64) for a in (x, y, z))
        _check(self._lib.gsq_sdf_eval(self._h, C.c_void_p(xs.ptr), C.c_void_p(ys.ptr), C.c_void_p(zs.ptr), 1,
                                      xs.n, C.c_void_p(_ptr(out)), None, None, _stream()))
        return out

    def compute_distances_tri(self, points, out=None):
        """Signed distances of (m, 3) points and each point's closest triangle
        (int32: c, or 2c / 2c + 1 within quad cell c; -1 for none), as a
        forward pass saves them for backward(..., dist=, triangles=)."""
        p = _Arr(points, np.float64, 3)
        m = p.n
        out = p.empty(m, np.float64) if out is None else out
        tri = p.empty(m, np.int32)
        base = p.ptr
        _check(self._lib.gsq_sdf_eval_tri(self._h, C.c_void_p(base), C.c_void_p(base + 8), C.c_void_p(base + 16), 3,
                                          m, C.c_void_p(_ptr(out)), C.c_void_p(_ptr(tri)), _stream()))
        return out, tri

    def backward(self, points, grad_dist, want_points: bool = True, want_vertices: bool = True, dist=None,
                 triangles=None):
        """Adjoint of compute_distances: (dL/dpoints (m,3), dL/dvertices (V,3)).
        With the forward's dist and triangles (compute_distances_tri) the
        closest triangles are not searched again."""
        p = _Arr(points, np.float64, 3)
        g = _Arr(grad_dist, np.float64)
        m = p.n
        gp = p.empty((m, 3), np.float64) if want_points else None
        gv = p.empty((self.num_vertices, 3), np.float64) if want_vertices else None
        base = p.ptr
        outs = (C.c_void_p(_ptr(gp)) if gp is not None else None, C.c_void_p(_ptr(gv)) if gv is not None else None)
        if triangles is not None:
            d = _Arr(dist, np.float64)
            t = _Arr(triangles, np.int32)
            _check(self._lib.gsq_sdf_backward_tri(self._h, C.c_void_p(base), C.c_void_p(base + 8),
                                                  C.c_void_p(base + 16), 3, m, C.c_void_p(d.ptr), C.c_void_p(t.ptr),
                                                  C.c_void_p(g.ptr), *outs, _stream()))
        else:
            _check(self._lib.gsq_sdf_backward(self._h, C.c_void_p(base), C.c_void_p(base + 8), C.c_void_p(base + 16),
                                              3, m, C.c_void_p(g.ptr), *outs, _stream()))
        return gp, gv

    def compute_distance(self, x: float, y: float, z: float) -> float:
        return float(self.compute_distances(np.array([[x, y, z]]))[0])

    def get_mesh_bounds(self):
        lo, hi = np.empty(3), np.empty(3)
        _check(self._lib.gsq_sdf_mesh_bounds(self._h, lo.ctypes.data_as(_dp), hi.ctypes.data_as(_dp)))
        return lo, hi

    def get_bvh_tree(self) -> BVH:
        b = _vp()
        _check(self._lib.gsq_sdf_get_bvh(self._h, C.byref(b)))
        return BVH(_handle=b)

    def last_eval_ms(self) -> float:
        v = C.c_float()
        _check(self._lib.gsq_sdf_last_eval_ms(self._h, C.byref(v)))
        return v.value


class Batch:
    """Many meshes, each with its own points, evaluated together (the batched
    form; no reference counterpart).  ``meshes`` is a list of (vertices (V_k, 3),
    cells (C_k, 3 or 4)) with mesh-local vertex ids; ``points`` a list of
    (M_k, 3) arrays.  Every run rebuilds all trees and evaluates all points
    with one CUDA graph launch; each mesh's results equal ``SignedDistance``
    on that mesh alone (MIXED or FP64: they agree bit for bit)."""

    def __init__(self, meshes, points, is_watertight: bool = True, compute_sign: bool = True,
                 closest_points: bool = False, **opts):
        self._lib = load()
        verts = [np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3) for v, _ in meshes]
        cells = [np.ascontiguousarray(c, dtype=np.int32) for _, c in meshes]
        npc = cells[0].shape[1]
        if any(c.shape[1] != npc for c in cells):
            raise ValueError("all meshes need the same nodes per cell")
        sizes = [int(np.asarray(p).reshape(-1, 3).shape[0]) if not _is_torch(p) else int(p.reshape(-1, 3).shape[0])
                 for p in points]
        self.vert_offsets = np.concatenate([[0], np.cumsum([v.shape[0] for v in verts])]).astype(np.int64)
        self.cell_offsets = np.concatenate([[0], np.cumsum([c.shape[0] for c in cells])]).astype(np.int64)
        self.point_offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.num_points = int(self.point_offsets[-1])
        allc = np.ascontiguousarray(np.concatenate(cells), dtype=np.int32)
        o = BatchOpts()
        _check(self._lib.gsq_batch_opts_init(C.byref(o)))
        for k, v in opts.items():
            setattr(o, k, int(v))
        o.closest_points = int(closest_points)
        h = _vp()
        _check(self._lib.gsq_batch_create(C.byref(h), len(meshes), C.c_void_p(self.vert_offsets.ctypes.data),
                                          C.c_void_p(self.cell_offsets.ctypes.data), C.c_void_p(allc.ctypes.data),
                                          npc, C.c_void_p(self.point_offsets.ctypes.data), int(is_watertight),
                                          int(compute_sign), C.byref(o), _stream()))
        self._h = h
        self.closest_points = closest_points
        self.set_vertices(np.concatenate(verts))
        self.set_points(points)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gsq_batch_destroy(self._h)
            self._h = None

    def set_vertices(self, vertices):
        """All meshes' vertices: a (sum V_k, 3) host array, or a tuple (x, y, z)
        of contiguous float64 arrays or tensors (host, pinned or device)."""
        if isinstance(vertices, tuple):
            xyz = [_Arr(a, np.float64) for a in vertices]
        else:
            v = np.ascontiguousarray(np.asarray(vertices, dtype=np.float64).reshape(-1, 3).T)
            xyz = [_Arr(v[k], np.float64) for k in range(3)]
        _check(self._lib.gsq_batch_set_vertices(self._h, *[C.c_void_p(a.ptr) for a in xyz], _stream()))

    def set_points(self, points):
        """A list of per-mesh (M_k, 3) arrays, or one (sum M_k, 3) array (host or device)."""
        if isinstance(points, (list, tuple)):
            if points and _is_torch(points[0]):
                import torch
                points = torch.cat([p.reshape(-1, 3) for p in points])
            else:
                points = np.concatenate([np.asarray(p, dtype=np.float64).reshape(-1, 3) for p in points])
        p = _Arr(points, np.float64, 3)
        if p.n != self.num_points:
            raise ValueError(f"expected {self.num_points} points, got {p.n}")
        self._points = p  # keeps a converted copy alive until the copy is done
        _check(self._lib.gsq_batch_set_points(self._h, C.c_void_p(p.ptr), _stream()))

    def run(self, out=None, closest=None):
        """Rebuilds every tree and evaluates every point.  Returns the distances
        (into ``out`` if given, else a new host array) and, if ``closest`` is
        True or an array, the closest points."""
        out = np.empty(self.num_points) if out is None else out
        if closest is True:
            closest = np.empty((self.num_points, 3))
        _check(self._lib.gsq_batch_run(self._h, C.c_void_p(_ptr(out)) if out is not False else None,
                                       C.c_void_p(_ptr(closest)) if closest is not None and closest is not False
                                       else None, _stream()))
        return (out, closest) if closest is not None and closest is not False else out

    def run_device(self):
        """Runs and leaves the results on the device; returns the last run's milliseconds."""
        _check(self._lib.gsq_batch_run(self._h, None, None, _stream()))
        return self.last_ms()

    def split(self, flat):
        """Per-mesh views of a flat per-point array."""
        return [flat[a:b] for a, b in zip(self.point_offsets[:-1], self.point_offsets[1:])]

    def tune(self) -> dict:
        _check(self._lib.gsq_batch_tune(self._h, _stream()))
        return self.opts()

    def opts(self) -> dict:
        o = BatchOpts()
        _check(self._lib.gsq_batch_get_opts(self._h, C.byref(o)))
        return o.as_dict()

    def set_opts(self, **kw):
        o = BatchOpts()
        _check(self._lib.gsq_batch_get_opts(self._h, C.byref(o)))
        for k, v in kw.items():
            setattr(o, k, int(v))
        _check(self._lib.gsq_batch_set_opts(self._h, C.byref(o)))

    def last_ms(self) -> float:
        v = C.c_float()
        _check(self._lib.gsq_batch_last_ms(self._h, C.byref(v)))
        return v.value

    def max_depth(self) -> int:
        v = C.c_int32()
        _check(self._lib.gsq_batch_max_depth(self._h, C.byref(v)))
        return v.value


class ClosestPoint:
    """The local closest-point query of quest::DistributedClosestPoint
    (quest/detail/DistributedClosestPointImpl.hpp:883-901, 1002-1050): a BVH
    over ``points`` (n, 3) with optional per-point ``domain_ids``, then for each
    query point the closest object point within ``distance_threshold``."""

    def __init__(self, points, domain_ids=None):
        self._lib = load()
        p = _Arr(points, np.float64, 3)
        d = _Arr(domain_ids, np.int32) if domain_ids is not None else None
        h = _vp()
        _check(self._lib.gsq_cpq_create(C.byref(h), C.c_void_p(p.ptr), p.n, C.c_void_p(d.ptr) if d else None,
                                        _stream()))
        self._h = h
        self.sq_threshold = float(np.finfo(np.float64).max)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.gsq_cpq_destroy(self._h)
            self._h = None

    def set_distance_threshold(self, t: float):
        """DistributedClosestPoint::setDistanceThreshold: stores t * t."""
        self.sq_threshold = float(t) * float(t)

    def compute_closest_points(self, queries, precision: int = PRECISION_MIXED):
        """(index (m,), domain (m,), position (m, 3), distance (m,)); -1 / NaN where none."""
        q = _Arr(queries, np.float64, 3)
        m = q.n
        idx, dom = q.empty(m, np.int32), q.empty(m, np.int32)
        pos, dist = q.empty((m, 3), np.float64), q.empty(m, np.float64)
        _check(self._lib.gsq_cpq_query(self._h, C.c_void_p(q.ptr), m, self.sq_threshold, precision,
                                       C.c_void_p(_ptr(idx)), C.c_void_p(_ptr(dom)), C.c_void_p(_ptr(pos)),
                                       C.c_void_p(_ptr(dist)), _stream()))
        return idx, dom, pos, dist

    def last_query_ms(self) -> float:
        v = C.c_float()
        _check(self._lib.gsq_cpq_last_ms(self._h, C.byref(v)))
        return v.value
