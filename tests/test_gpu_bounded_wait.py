"""GPU: a bounded wait that runs out is reported as an error, the kernel ends
and the context stays usable.

gsq_selftest_bounded_wait runs one block of the radix sort's onesweep pass on
the second tile of a two-tile input while the first tile is never processed:
its decoupled look-back waits for a flag that nothing sets.  No fault is
involved: the wait gives up after its poll limit, the block finishes its pass
inside its buffers, and the device error word carries DEVERR_WAIT, which the
call reports as GSQ_ERR_DEVICE.  A build and a find run right after it give
the oracle's answer.
"""
from __future__ import annotations

import time

import numpy as np
import pytest

from axom_gb300 import workloads as W
from conftest import assert_bits_equal

pytestmark = pytest.mark.gpu

GSQ_ERR_DEVICE = -4


def test_expired_lookback_wait_is_reported(gsq, port):
    lib = gsq.load()
    t0 = time.perf_counter()
    rc = lib.gsq_selftest_bounded_wait(None)
    seconds = time.perf_counter() - t0
    assert rc == GSQ_ERR_DEVICE
    assert "expired bounded wait" in lib.gsq_last_error().decode()
    assert seconds < 60.0, seconds
    print(f"the expired wait took {seconds:.2f} s")
    # the context is usable: a build and a find equal the oracle's
    boxes = W.random_boxes(20_000, 21)
    q = W.random_boxes(2_000, 22)
    b = gsq.BVH(boxes)
    h = port.bvh(boxes)
    for x, y, what in zip(b.find_bounding_boxes(q), port.find_boxes(h, q), ("offsets", "counts", "candidates")):
        assert_bits_equal(np.asarray(x), y, what)
