"""The C++ drop-in layer run on the GPU: the reference's known answers through
spgemm_gb300::spgemm and spgemm_gb300::LocalAccumulator with the reference's
CsrMatrix layout and exception types (tests/cpp/shim_test.cpp)."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_cpp_shim(tmp_path):
    lib_dir = ROOT / "spgemm-hpc-thesis_gb300"
    exe = tmp_path / "shim_test"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "shim_test.cpp"),
                    f"-L{lib_dir}", "-lspgemm_gb300", "-o", str(exe)], check=True)
    env = dict(os.environ, LD_LIBRARY_PATH=f"{lib_dir}:{os.environ.get('LD_LIBRARY_PATH', '')}")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASS" in r.stdout
