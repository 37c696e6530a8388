"""The quest signed-distance interface for Python, with the functions of the
reference's Python module (quest/interface/python/pyQUESTmodule.cpp, the
shroud binding of quest/interface/signed_distance.hpp:88-319): a global query
object built from an STL file, evaluated one point at a time, on the GPU
through the QUEST_signed_distance_* entry points of libgsq.so
(include/gsq_quest.h).

As in the reference, options are set before ``signed_distance_init``, and
misuse (an option after init, evaluate before init, a dimension other than 3)
aborts the process.  ``signed_distance_evaluate(x, y, z)`` returns the signed
distance; with the six extra arguments of the reference's second form it
returns ``(phi, cp_x, cp_y, cp_z, n_x, n_y, n_z)`` (the extra arguments are
ignored, as they are outputs there).  ``signed_distance_evaluate_points`` and
``signed_distance_get_mesh_bounds`` add the array form and the bounds of
signed_distance.hpp:290 and :308, which the reference's Python module lacks.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import load

SignedDistExec_CPU = 0
SignedDistExec_OpenMP = 1
SignedDistExec_GPU = 2


def signed_distance_init(file: str) -> int:
    """0 on success, -1 when the file cannot be read or the query built."""
    return load().QUEST_signed_distance_init_serial(str(file).encode())


def signed_distance_initialized() -> bool:
    return bool(load().QUEST_signed_distance_initialized())


def signed_distance_set_dimension(dim: int) -> None:
    load().QUEST_signed_distance_set_dimension(int(dim))


def signed_distance_set_closed_surface(status: bool) -> None:
    load().QUEST_signed_distance_set_closed_surface(bool(status))


def signed_distance_set_compute_signs(computeSign: bool) -> None:
    load().QUEST_signed_distance_set_compute_signs(bool(computeSign))


def signed_distance_set_allocator(allocatorID: int) -> None:
    load().QUEST_signed_distance_set_allocator(int(allocatorID))


def signed_distance_set_verbose(status: bool) -> None:
    load().QUEST_signed_distance_set_verbose(bool(status))


def signed_distance_use_shared_memory(status: bool) -> None:
    load().QUEST_signed_distance_use_shared_memory(bool(status))


def signed_distance_set_execution_space(execSpace: int) -> None:
    load().QUEST_signed_distance_set_execution_space(int(execSpace))


def signed_distance_evaluate(x, y, z, *outputs):
    """phi, or (phi, cp_x, cp_y, cp_z, n_x, n_y, n_z) when called with the six
    output arguments of the reference's second form."""
    lib = load()
    if not outputs:
        return lib.QUEST_signed_distance_evaluate_0(float(x), float(y), float(z))
    if len(outputs) != 6:
        raise TypeError("signed_distance_evaluate takes 3 or 9 arguments")
    o = [C.c_double() for _ in range(6)]
    phi = lib.QUEST_signed_distance_evaluate_1(float(x), float(y), float(z), *[C.byref(v) for v in o])
    return (phi,) + tuple(v.value for v in o)


def signed_distance_evaluate_points(x, y, z) -> np.ndarray:
    """The array form (signed_distance.hpp:290) over three coordinate arrays."""
    xs, ys, zs = (np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (x, y, z))
    if not (xs.size == ys.size == zs.size):
        raise ValueError("x, y and z differ in length")
    phi = np.empty(xs.size)
    load().gsq_quest_evaluate_points(xs.ctypes.data, ys.ctypes.data, zs.ctypes.data, xs.size, phi.ctypes.data)
    return phi


def signed_distance_get_mesh_bounds() -> tuple[np.ndarray, np.ndarray]:
    lo, hi = (C.c_double * 3)(), (C.c_double * 3)()
    load().QUEST_signed_distance_get_mesh_bounds(lo, hi)
    return np.array(lo[:]), np.array(hi[:])


def signed_distance_finalize() -> None:
    load().QUEST_signed_distance_finalize()
