"""The FP32 node-visit certificate of the mixed signed distance
(axom_gb300/csrc/gsq_leaf32.cuh: node_box32, qctx_init / qctx_set32,
box_decide and visit32_core, the code the query kernels run), checked on the
host against the FP64 visit of the oracle (squared_distance(Point,
BoundingBox) <= minSq per child and the nearer-centroid-first order,
policy/LinearBVH.hpp:72-85) and exact long-double values: a certified visit
enters a child only if every minSq of the context's interval admits it,
excludes it only if none does, and orders two entered children as the FP64
centroid comparison does, with or without fused products.  Random boxes
(flat, invalid, sharing a face, nested), points on faces, inside, just off a
face and far away, mirror-image siblings whose centroids are all but
equidistant from the point, and intervals on a child's own distance."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def node_check(tmp_path_factory):
    exe = tmp_path_factory.mktemp("node") / "node_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", str(ROOT / "tests/cpp/node_check.cpp"), "-o",
                    str(exe)], check=True)
    return exe


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_node_certificate_decisions(node_check, mode):
    r = subprocess.run([str(node_check), "1000000", str(41 + mode), str(mode)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    words = r.stdout.split("|")[0].split()
    count = {words[i]: int(words[i + 1]) for i in range(0, len(words) - 1) if words[i + 1].isdigit()}
    # the certificate decides a share of these adversarial visits (intervals
    # placed on a child's own distance) and both orders occur
    assert count["certified"] > 50000 and count["both"] > 0 and 0 < count["swaps"] < count["both"], r.stdout
