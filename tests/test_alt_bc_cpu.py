"""Alternate boundaries against the reference's own per-cell functions.

Fixtures (tests/golden/alt_bc.npz, made by tests/golden/make_golden.py) hold
the reference's outputs on seeded near-equilibrium cells at every edge and
corner class of its domain:
  CPU_3D/CPU_3D.cpp boundaries() (CPU:1027-1078): 3 DirichletWest,
    13 DirichletWest_Reg, 14 NeumannEast_Reg, 54 NeumannEast_Regularized, 21/22 ysymmetry_top/_bot,
    23/24 zsymmetry_top/_bot, on its 43 x 43 face with UMAX = 0.04, and
    its DirichletNorth_Reg / DirichletSouth_Reg (CPU:578-745);
  LRTurbTest/LRMultiGPU7.cu xsymmetry_top / _bot (LR7:899-1016);
  BC1/LRMultiGPU7.cu West_Reg (:789-870) at perturbed and plain steps.
The product's cell functions (host build of d3q19.cuh) and the oracle's
restatement must reproduce the copies and closed forms bit for bit.  West_Reg
is the exception: the reference rebuilds all 19 populations from their MRT
moments with the momenta replaced, which equals the momentum-only update
f += c . (j_target - j) / 10 exactly in real arithmetic; the two FP32
evaluations differ by rounding, so that case uses the per-cell FP32
tolerance of the collide tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle_bindings import ref_lib

P = ctypes.c_void_p
F = ctypes.c_float

NODE = dict(DIR_WEST=8, NEU_EAST=9, NEU_EAST_REG=10, XSYM_TOP=11, XSYM_BOT=12, YSYM_TOP=13, YSYM_BOT=14,
            ZSYM_TOP=15, ZSYM_BOT=16, WEST_REG=17, DIR_WEST_V=18, DIR_NORTH=19, DIR_SOUTH=20)
# FP32 per-cell tolerance (populations O(0.03..0.33)); the same bound as the
# collide tests, for a map the reference evaluates in another order
ATOL_CELL = 5e-7
CPU3D_CODE = {3: "DIR_WEST", 13: "DIR_WEST_V", 14: "NEU_EAST", 54: "NEU_EAST_REG", 21: "YSYM_TOP", 22: "YSYM_BOT",
              23: "ZSYM_TOP", 24: "ZSYM_BOT"}


def ptr(a):
    return a.ctypes.data_as(P)


@pytest.fixture(scope="module")
def alt(golden):
    return np.load(golden["dir"] / "alt_bc.npz")


def run(lib_fn, kind, f0, yz, dims, u, t):
    g = np.ascontiguousarray(f0, np.float32).copy()
    lib_fn(NODE[kind], ptr(g), len(g), ptr(np.ascontiguousarray(yz, np.int32)), int(dims[0]), int(dims[1]),
           F(u), int(t))
    return g


def test_product_node_codes_match_the_oracle(product):
    """the package's node codes, the oracle header's and the ones these tests use agree"""
    import re

    from oracle_bindings import ref_recipe

    hdr = (ref_recipe.HERE / "lbm_oracle.h").read_text()
    for k, v in NODE.items():
        assert product.NODE[k] == v
        assert re.search(rf"ORC_{k}\s*=\s*{v}\b", hdr), k


@pytest.mark.parametrize("im", sorted(CPU3D_CODE))
def test_cpu3d_boundaries_vs_reference(alt, cellops, orc, im):
    kind = CPU3D_CODE[im]
    f0, yz, dims, u = alt["cpu3d_f0"], alt["cpu3d_yz"], alt["cpu3d_dims"], float(alt["cpu3d_umax"])
    want = alt[f"cpu3d_im{im}"]
    assert not np.array_equal(want, f0)
    for fn in (cellops.cell_alt_boundary, orc.orc_alt_boundary):
        got = run(fn, kind, f0, yz, dims, u, 0)
        np.testing.assert_array_equal(got, want, err_msg=f"{kind} (CPU_3D im {im})")


@pytest.mark.parametrize("north", [1, 0])
def test_cpu3d_moving_walls_vs_reference(alt, cellops, orc, north):
    f0, yz, dims, u = alt["cpu3d_f0"], alt["cpu3d_yz"], alt["cpu3d_dims"], float(alt["cpu3d_umax"])
    want = alt[f"cpu3d_dirichlet_north{north}"]
    for fn in (cellops.cell_alt_boundary, orc.orc_alt_boundary):
        got = run(fn, "DIR_NORTH" if north else "DIR_SOUTH", f0, yz, dims, u, 0)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("top", [1, 0])
def test_lr7_xsymmetry_vs_reference(alt, cellops, orc, top):
    f0, yz, dims = alt["lr7_f0"], alt["lr7_yz"], alt["lr7_dims"]
    want = alt[f"lr7_xsym_top{top}"]
    for fn in (cellops.cell_alt_boundary, orc.orc_alt_boundary):
        got = run(fn, "XSYM_TOP" if top else "XSYM_BOT", f0, yz, dims, 0.0, 0)
        np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("t", [1, 1000, 2000, 3000, 4000])
def test_bc1_west_reg_vs_reference(alt, cellops, orc, t):
    f0 = alt["bc1_f0"]
    want = alt[f"bc1_west_reg_u0.05_t{t}"]
    yz = np.zeros((len(f0), 2), np.int32)
    for fn in (cellops.cell_alt_boundary, orc.orc_alt_boundary):
        got = run(fn, "WEST_REG", f0, yz, (8, 8), 0.05, t)
        np.testing.assert_allclose(got, want, atol=ATOL_CELL, rtol=0)


def test_fixtures_match_the_reference_build(alt):
    """where the staged reference harness is present, the committed fixtures
    are still what it produces"""
    c3 = ref_lib("cpu3d.so")
    if c3 is None:
        pytest.skip("reference harness not staged")
    f0, yz = alt["cpu3d_f0"], alt["cpu3d_yz"]
    for im in CPU3D_CODE:
        g = f0.copy()
        c3.ref_cpu3d_boundary(ptr(g), len(g), ptr(yz), im)
        np.testing.assert_array_equal(g, alt[f"cpu3d_im{im}"])


def test_west_reg_sets_the_momentum(alt, cellops):
    """West_Reg's map f += c . (j_target - j) / 10 sets the momentum to
    (u, 0, w) (sum_q c_x^2 = 10 on D3Q19) and keeps rho"""
    from oracle_bindings import CX, CY, CZ

    f0 = alt["bc1_f0"].astype(np.float32)
    yz = np.zeros((len(f0), 2), np.int32)
    g = run(cellops.cell_alt_boundary, "WEST_REG", f0, yz, (8, 8), 0.05, 1000)
    a, b = f0.astype(np.float64), g.astype(np.float64)
    np.testing.assert_allclose(b.sum(1), a.sum(1), atol=1e-6)
    for c, target in ((CX, 0.05), (CY, 0.0), (CZ, 0.01)):
        np.testing.assert_allclose(b @ c, target, rtol=0, atol=2e-6)
