"""The C++ drop-in layer compiles against the reference's own CsrMatrix
(src/common/csr_matrix.hpp) and instantiates the trident::LocalAccumulator
substitution, where the reference tree is present (REFERENCE_ROOT, else a
``reference`` directory beside the repository); skipped elsewhere.  Running
the same program needs a GPU (test_gpu_cpp_dropin.py)."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_shim_compiles_against_reference_csr():
    from oracle import build as obuild
    common = obuild.reference_root() / "src" / "common"
    if not (common / "csr_matrix.hpp").exists():
        pytest.skip("reference tree not present")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-DSPG_REFERENCE_CSR", f"-I{ROOT / 'include'}",
                        f"-I{common}", str(ROOT / "tests" / "cpp" / "shim_test.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
