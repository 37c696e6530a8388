"""The FP32 certificate of the signed distance's sign (axom_gb300/csrc/gsq_sign.cuh,
used by the mixed query kernel when no normals are written), checked on the host
against the oracle's FP64 sign test (the reference's computeSign with its face
normal or pseudo-normal sum): random faces, vertex fans with slivers and
degenerate triangles, and shared edges, with query points from along the normal
down to nearly tangent, at 1e-9..10 times the triangle size.  Whenever the
certificate gives a sign it must be the FP64 test's."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def sign_check(tmp_path_factory):
    exe = tmp_path_factory.mktemp("sign") / "sign_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", str(ROOT / "tests/cpp/sign_check.cpp"),
                    "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("seed,mode,share", [(1, 0, 0.75), (2, 0, 0.75), (3, 1, 0.5)])
def test_sign_certificate_agrees_with_fp64(sign_check, seed, mode, share):
    """mode 1: the same cases at coordinates up to 1e3, where the rounding of
    the vertices weighs more and fewer signs are certified."""
    r = subprocess.run([str(sign_check), "1500000", str(seed), str(mode)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    # the certificate must also decide most cases (else the FP64 path does the work)
    fields = r.stdout.split("|")[0].split()
    for name in ("face", "vertex", "edge"):
        done, total = map(int, fields[fields.index(name) + 1].split("/"))
        assert done >= share * total, r.stdout
