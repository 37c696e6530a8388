"""GPU: a C++ program written against include/gsq.hpp (the reference-named
shim) compiles with g++, links libgsq.so and passes the reference's
known-answer checks."""
from __future__ import annotations

import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_cpp_shim_known_answers(gsq, tmp_path):
    exe = tmp_path / "shim_check"
    lib_dir = ROOT / "axom_gb300"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/shim_check.cpp"),
                    f"-L{lib_dir}", "-lgsq", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    p = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, cwd=tmp_path)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "OK" in p.stdout
