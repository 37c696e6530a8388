"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    """The C++ restatement of the reference (the oracle)."""
    import oracle
    return oracle.Port()


@pytest.fixture(scope="session")
def ref():
    """The reference's own SEQ code, where it could be built from its sources."""
    import oracle
    if not oracle.ref_available():
        try:
            if oracle.build_reference() is None:
                pytest.skip("reference sources not present")
        except Exception as e:  # pragma: no cover - depends on the host
            pytest.skip(f"reference could not be built: {e}")
    return oracle.Ref()


@pytest.fixture(scope="session")
def gsq():
    """The product library on the GPU; fails loudly if it cannot be loaded."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from axom_gb300 import build
    build.build()
    import axom_gb300
    axom_gb300.load()
    torch.cuda.init()
    return axom_gb300


def golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def assert_bits_equal(a, b, what=""):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if not np.array_equal(a.view(np.uint8), b.view(np.uint8)):
        diff = np.flatnonzero((a != b).reshape(-1) if a.dtype.kind != "f" else
                              (a.view(np.int64 if a.itemsize == 8 else np.int32) !=
                               b.view(np.int64 if b.itemsize == 8 else np.int32)).reshape(-1))
        raise AssertionError(f"{what}: {diff.size} entries differ, first at {diff[:5]}: "
                             f"{a.reshape(-1)[diff[:5]]} vs {b.reshape(-1)[diff[:5]]}")


def csr_sets(off, cnt, cand):
    return [tuple(sorted(cand[o:o + c])) for o, c in zip(off, cnt)]
