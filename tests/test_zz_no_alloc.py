"""GPU: the allocation-free entry point gsq_sdf_eval_noalloc.

It exists for callers that must not allocate device memory while they
evaluate (an application whose pool allocator owns all device memory, or
other streams that must not be stalled by cudaMalloc's device-wide
synchronisation).  Its only scratch is a fixed array in the
library's device image shared by all calls, so this test calls it twice in a
row on different point sets and checks each call against gsq_sdf_eval, with
the tolerance the other signed-distance tests use (bit-exact distances).  It
is collected last and passes alone in a fresh process as well as after the
rest of the suite.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, sd, q_dev, out_dev):
    import torch
    base = q_dev.data_ptr()
    rc = lib.gsq_sdf_eval_noalloc(sd._h, C.c_void_p(base), C.c_void_p(base + 8), C.c_void_p(base + 16), 3,
                                  q_dev.shape[0], C.c_void_p(out_dev.data_ptr()),
                                  C.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_eval_twice(gsq, precision):
    import torch
    from axom_gb300 import workloads as W
    lib = gsq.load()
    v, f = W.displaced_icosphere(6, 21)
    sd = gsq.SignedDistance(v, f, precision=precision)
    for call, (m, seed) in enumerate(((gsq.NOALLOC_MAX_QUERIES, 5), (70001, 6))):
        q = torch.from_numpy(W.mixed_queries(v, f, m, seed)).cuda()
        ref = sd.compute_distances(q)
        out = torch.full((m,), float("nan"), dtype=torch.float64, device="cuda")
        assert _noalloc(lib, sd, q, out) == 0, lib.gsq_last_error()
        torch.cuda.synchronize()
        assert torch.equal(out.view(torch.int64), ref.view(torch.int64)), f"call {call} differs"


def test_noalloc_rejects_oversize_and_host_memory(gsq):
    import torch
    from axom_gb300 import workloads as W
    lib = gsq.load()
    v, f = W.displaced_icosphere(3, 1)
    sd = gsq.SignedDistance(v, f)
    m = gsq.NOALLOC_MAX_QUERIES + 1
    q = torch.zeros((m, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(m, dtype=torch.float64, device="cuda")
    assert _noalloc(lib, sd, q, out) == -1
    assert b"GSQ_NOALLOC_MAX_QUERIES" in lib.gsq_last_error()
    qh = np.zeros((4, 3))
    oh = np.zeros(4)
    rc = lib.gsq_sdf_eval_noalloc(sd._h, C.c_void_p(qh.ctypes.data), C.c_void_p(qh.ctypes.data + 8),
                                  C.c_void_p(qh.ctypes.data + 16), 3, 4, C.c_void_p(oh.ctypes.data), None)
    assert rc == -1 and b"device memory" in lib.gsq_last_error()
