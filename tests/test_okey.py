"""The exact FP64 comparisons on the integer pipe (axom_gb300/csrc/
gsq_internal.cuh: okey with ok_lt / ok_gt / ok_le / ok_ge / ok_eq and
box_valid_k, and gt_eps / lt_neg_eps / abs_le_eps for closest_point's fuzzy
tests), which the BVH build, the candidate queries and the signed-distance
kernels use in place of FP64 comparisons, checked on the host against the IEEE
comparisons: special values (signed zeros, subnormals, extremes, infinities,
NaNs of either sign and any payload) and 5M random pairs of bit patterns
(unrelated, adjacent, one bit apart, sharing the high word)."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def okey_check(tmp_path_factory):
    from axom_gb300 import build
    cuda_inc = Path(build.nvcc()).resolve().parents[1] / "include"
    exe = tmp_path_factory.mktemp("okey") / "okey_check"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{cuda_inc}", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests/cpp/okey_check.cpp"), "-o", str(exe)], check=True)
    return exe


def test_integer_pipe_comparisons_equal_ieee(okey_check):
    r = subprocess.run([str(okey_check), "5000000", "17"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
