"""The FP32 enclosure of a query-to-object-point squared distance used by the
mixed closest-point kernel (axom_gb300/csrc/gsq_leaf32.cuh: qctx_init and
point_bounds32, the code the kernel runs), checked on the host against the
FP64 squared distance of the oracle (squared_distance(Point, Point),
primal/operators/squared_distance.hpp:62-67) and its exact long-double value:
the FP64 value lies inside the enclosure in every case.  Unit-sized scenes,
coordinates up to 1e3 with nearby points, points within 1e-20..1e-5 of the
query or on it, and queries up to 1e2 away."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def point_check(tmp_path_factory):
    exe = tmp_path_factory.mktemp("point") / "point_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(ROOT / "tests/cpp/point_check.cpp"), "-o",
                    str(exe)], check=True)
    return exe


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_point_enclosure_holds(point_check, mode):
    r = subprocess.run([str(point_check), "1000000", str(61 + mode), str(mode)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split("|")[0].split()
    count = {words[i]: int(words[i + 1]) for i in range(0, len(words) - 1) if words[i + 1].isdigit()}
    assert count["violations"] == 0
    if mode in (0, 3):  # away from coincidence the enclosure is tight enough to decide
        assert count["tight"] > 990000, r.stdout
