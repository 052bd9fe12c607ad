"""Test configuration.

Markers: ``gpu`` -- needs a CUDA device (run with ``-m gpu``); everything
else runs on the CPU. The CUDA library and the CPU oracle are built on
first use if they are missing (nvcc cross-compiles without a GPU).
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    from fluids3_gb300 import build as B
    B.build()
    from oracle import oracle as O
    srcs = [O.HERE / "fluids_oracle.c", O.HERE / "adjoint64.c", O.HERE / "build_oracle.sh"]
    if not O.ORACLE_LIB.exists() or any(f.stat().st_mtime > O.ORACLE_LIB.stat().st_mtime for f in srcs):
        O.build(ref=False)


_ensure_built()


@pytest.fixture(scope="session")
def golden_dir() -> Path:
    return ROOT / "tests" / "golden"
