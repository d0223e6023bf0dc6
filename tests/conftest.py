"""pytest configuration: the `gpu` marker and session fixtures that build the
product library, the oracle and the test-only host build of the product's
per-cell operators."""
from __future__ import annotations

import ctypes
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "tests", ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # the tests' temporary files stay inside the working tree (git-ignored)
    if not config.option.basetemp:
        config.option.basetemp = str(ROOT / ".pytest_tmp")


@pytest.fixture(scope="session")
def product():
    """the product package with its CUDA library built in-tree"""
    from lbm_multigpu_gb300 import build

    build.build()
    import lbm_multigpu_gb300 as lbm

    lbm.library()
    return lbm


@pytest.fixture(scope="session")
def orc():
    from oracle_bindings import oracle

    return oracle()


@pytest.fixture(scope="session")
def cellops(tmp_path_factory):
    """host build of lbm_multigpu_gb300/csrc/d3q19.cuh (test-only shim)"""
    from lbm_multigpu_gb300.build import nvcc

    out = tmp_path_factory.mktemp("cellops") / "cellops.so"
    src = ROOT / "tests" / "native" / "cell_ops_shim.cu"
    r = subprocess.run([nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared", "-o",
                        str(out), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(str(out))
    lib.cell_philox_uniform.restype = ctypes.c_float
    return lib


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    import json

    g = ROOT / "tests" / "golden"
    runs, meta = {}, {}
    for stem in ("runs", "runs_1k"):  # the 1000-step channel is its own file
        runs.update(dict(np.load(g / f"{stem}.npz")))
        meta.update(json.loads((g / f"{stem}.json").read_text()))
    return dict(cells=np.load(g / "cells.npz"), runs=runs, meta=meta, dir=g)
