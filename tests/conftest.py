"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the built
engine; everything else runs on the CPU (oracle, golden vectors, host logic,
C-ABI exports)."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "spgemm-hpc-thesis_gb300"
for p in (str(ROOT), str(PKG), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA engine")


@pytest.fixture(scope="session")
def port():
    from oracle import build as obuild
    from oracle.oracle import Port
    obuild.build_oracle()
    return Port()


@pytest.fixture(scope="session")
def engine():
    import spgemm_gb300 as sg
    eng = sg.Engine(0)
    yield eng
    eng.close()
