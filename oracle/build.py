"""Build recipe for the CPU checkers under oracle/ (test infrastructure only).

* ``build_oracle()`` compiles the C++ restatement ``spgemm_oracle.cpp`` into
  ``oracle/liboracle.so``.  It runs on every host (the GPU hosts included).
* ``build_ref()`` compiles the reference's own local-multiply sources, in place
  from the read-only reference tree, together with ``ref_shim.cpp`` and the
  single-rank ``ref_stub/mpi.h``, into ``oracle/_ref/libspgemm_ref.so``.  It
  needs the reference checkout: ``REFERENCE_ROOT``, else a ``reference``
  directory beside the repository; it is skipped where that tree is absent.

Both libraries use -O3 -fopenmp -ffp-contract=off: the reference source
multiplies and adds in separate statements, and the checkers keep those two
roundings on every architecture.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_SO = REF_DIR / "libspgemm_ref.so"

# The reference files that hold the local multiply, its serial twin, the
# uncached Partial/Full validators, the Trident accumulator and the MTX reader.
REF_SOURCES = [
    "src/common/spgemm_common.cpp",
    "src/common/matrix_market.cpp",
    "src/baselines/spgemm_exchange.cpp",
    "src/trident/common/matrix_blocks.cpp",
    "src/trident/common/process_grid.cpp",
]
REF_INCLUDES = ["src/common", "src/baselines", "src/trident/common"]
FLAGS = ["-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17"]


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> Path:
    src = HERE / "spgemm_oracle.cpp"
    if force or _stale(ORACLE_SO, [src]):
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        subprocess.run(["g++", *FLAGS, str(src), "-o", str(tmp)], check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_root() -> Path:
    env = os.environ.get("REFERENCE_ROOT")
    return Path(env) if env else HERE.parents[1] / "reference"


def build_ref(force: bool = False) -> Path | None:
    root = reference_root()
    if not (root / REF_SOURCES[0]).exists():
        return None
    sources = [root / s for s in REF_SOURCES]
    shim = HERE / "ref_shim.cpp"
    stub = HERE / "ref_stub" / "mpi.h"
    if force or _stale(REF_SO, sources + [shim, stub]):
        REF_DIR.mkdir(exist_ok=True)
        incs = [f"-I{HERE / 'ref_stub'}"] + [f"-I{root / i}" for i in REF_INCLUDES]
        tmp = REF_SO.with_suffix(".so.tmp")
        subprocess.run(["g++", *FLAGS, "-w", *incs, *map(str, sources), str(shim), "-o", str(tmp)],
                       check=True)
        os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
