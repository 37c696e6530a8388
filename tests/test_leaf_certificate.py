"""The FP32 leaf certificate of the mixed signed distance
(axom_gb300/csrc/gsq_leaf32.cuh: the leaf records' error terms, the query
context and tri_bounds, the code the query kernels run), checked on the host
against the oracle's FP64 closest_point (the reference's algorithm, fuzzy
comparisons included) and an exact long-double distance: a skipped
triangle's FP64 distance exceeds the threshold, a kept triangle's FP64 squared
distance lies in [l2, h2], and its FP64 closest point lies within rad of the
estimate.  Random triangles of mixed sizes, slivers (kappa up to 2^20),
coordinates up to 1e3, tiny triangles (also at coordinates up to 1e3) and
distant points; quads' triangles too."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def leaf_check(tmp_path_factory):
    exe = tmp_path_factory.mktemp("leaf") / "leaf_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", str(ROOT / "tests/cpp/leaf_check.cpp"),
                    "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4])
def test_leaf_certificate_bounds(leaf_check, mode):
    r = subprocess.run([str(leaf_check), "1000000", str(31 + mode), str(mode)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    counts = r.stdout.split("|")[0].split()
    assert int(counts[counts.index("skipped") + 1]) > 0 and int(counts[counts.index("kept") + 1]) > 0, r.stdout


def test_leaf_certificate_sliver_thinner_than_rounding(leaf_check):
    """Seed 901 of mode 1 draws a quad's sliver 6.7e-7 wide at coordinates
    near 44, whose FP32 vertices move by 4.5e-6: the rounded triangle is far
    thinner than the FP64 one, and a conditioning factor taken from the FP64
    triangle let the certificate skip it at an FP64 distance of 5.7e-7.
    Triangles narrower than 64 times their vertices' rounding are never
    skipped now."""
    r = subprocess.run([str(leaf_check), "5000000", "901", "1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
