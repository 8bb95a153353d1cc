"""The C ABI library without a GPU: it loads, exports every function that
include/*.h declares, reports statuses by name, and refuses to start (rather
than falling back to the CPU) where no CUDA device exists.  The C++ drop-in
header compiles against it."""
from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"


def declared_functions() -> list[str]:
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(spg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    import spgemm_gb300 as sg
    import build as engine_build
    engine_build.build()
    return sg.library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(lib):
    lib.spg_status_string.restype = C.c_char_p
    assert lib.spg_status_string(0) == b"SPG_OK"
    assert lib.spg_status_string(3) == b"SPG_OUT_OF_RANGE_COLUMN"
    assert lib.spg_status_string(9) == b"SPG_CANCELLED"


def test_null_arguments_rejected(lib):
    assert lib.spg_create(None, None) == 1
    assert lib.spg_multiply(None, None, None, 0, None) == 1
    assert lib.spg_config_default(None) == 1


def test_no_gpu_no_fallback(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    import spgemm_gb300 as sg
    with pytest.raises(sg.SpgError) as e:
        sg.Engine(0)
    assert e.value.name == "SPG_CUDA_ERROR"


def test_cpp_dropin_header_compiles(tmp_path, lib):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    out = tmp_path / "shim_test"
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", f"-I{INCLUDE}",
                        str(ROOT / "tests" / "cpp" / "shim_test.cpp"), f"-L{ROOT / 'spgemm-hpc-thesis_gb300'}",
                        "-lspgemm_gb300", "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
