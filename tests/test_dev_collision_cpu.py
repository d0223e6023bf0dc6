"""The projected MRT collision on stored deviations (collide_mrt_dev, the
FP16 / BF16 storage path of the stream-collide kernel) against LR7's MRT
collision (collide_mrt<MRT>, LRTurbTest/LRMultiGPU7.cu:583-711) applied to
the full populations, on the host build of the per-cell operators.

The deviations are taken from the model's own equilibrium at density 1 and
the reference velocity (U, 0, 0), which is what the FP16 / BF16 levels store
as offsets; that equilibrium is the MRT collision at omega = 1 of any state
with that density and momentum."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from oracle_bindings import CX, CY, CZ, W

MRT = 0


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _feq_bgk(rho, u):
    cu = CX * u[0] + CY * u[1] + CZ * u[2]
    return W * (rho + 3 * cu + 4.5 * cu ** 2 - 1.5 * float(np.dot(u, u)))


def _model_eq(cellops, u):
    f = _feq_bgk(1.0, np.array([u, 0.0, 0.0])).astype(np.float64).copy()
    cellops.cell_collide_d(MRT, 0, ctypes.c_double(1.0), ctypes.c_double(0.0), ctypes.c_double(0.0), _ptr(f), 1)
    return f


def _states(off, n, seed, amp):
    """populations near a sheared flow: equilibria at random density and
    velocity plus a random non-equilibrium part"""
    rng = np.random.default_rng(seed)
    f = np.empty((n, 19))
    for i in range(n):
        rho = 1 + rng.uniform(-0.02, 0.02)
        u = rng.uniform(-0.08, 0.08, 3)
        f[i] = _feq_bgk(rho, u) + amp * W * rng.standard_normal(19)
    return f, f - off


@pytest.mark.parametrize("les", [0, 1])
@pytest.mark.parametrize("u", [0.0, 0.05])
def test_dev_collision_equals_mrt_in_fp64(cellops, les, u):
    off = _model_eq(cellops, u)
    f, h = _states(off, 400, 1 + les, 0.01)
    om, cs = 1 / 0.52, 0.01
    cellops.cell_collide_d(MRT, les, ctypes.c_double(om), ctypes.c_double(cs), ctypes.c_double(0.0), _ptr(f), len(f))
    cellops.cell_collide_mrt_dev_d(les, ctypes.c_double(om), ctypes.c_double(cs), ctypes.c_double(u), _ptr(h), len(h))
    # collide_mrt rounds 2/3 to 0.666666667 (as LR7 writes it): ~1e-12 apart
    np.testing.assert_allclose(h + off, f, rtol=0, atol=1e-11)


def test_dev_collision_fp32_within_rounding(cellops):
    """in FP32 the deviation form is as accurate as the full-population form:
    both within a few ulp of 1 of the FP64 result"""
    u = 0.05
    off = _model_eq(cellops, u)
    f64, h64 = _states(off, 400, 7, 0.01)
    om, cs = 1 / 0.52, 0.01
    ref = f64.copy()
    cellops.cell_collide_d(MRT, 1, ctypes.c_double(om), ctypes.c_double(cs), ctypes.c_double(0.0), _ptr(ref), len(ref))
    f32 = f64.astype(np.float32)
    h32 = h64.astype(np.float32)
    cellops.cell_collide(MRT, 1, ctypes.c_float(om), ctypes.c_float(cs), ctypes.c_float(0.0), _ptr(f32), len(f32))
    cellops.cell_collide_mrt_dev(1, ctypes.c_float(om), ctypes.c_float(cs), ctypes.c_float(u), _ptr(h32), len(h32))
    e_full = np.abs(f32 - ref).max()
    e_dev = np.abs(h32.astype(np.float64) + off - ref).max()
    assert e_full < 5e-7 and e_dev < 5e-7, (e_full, e_dev)


def test_model_equilibrium_is_a_fixed_point(cellops):
    """the stored offsets of an LR7-MRT level are a steady state of the
    collision (zero deviation stays zero), and differ from the lattice
    weights by LR7's m2 equilibrium (7.54 j^2 instead of 3 rho - 11/2 j^2)"""
    u = 0.05
    off = _model_eq(cellops, u)
    h = np.zeros((1, 19))
    cellops.cell_collide_mrt_dev_d(1, ctypes.c_double(1 / 0.52), ctypes.c_double(0.01), ctypes.c_double(u), _ptr(h), 1)
    assert np.abs(h).max() < 1e-16
    assert abs(off.sum() - 1) < 1e-14 and abs(float(np.dot(CX, off)) - u) < 1e-14
    assert off[0] < 0.2  # 4/21 at rest, not the weight 1/3


@pytest.mark.parametrize("les", [0, 1])
def test_projected_collision_on_full_populations(cellops, les):
    """with U = 0 the projected collision takes full populations (the
    closure kernel's FP32 path): it equals collide_mrt<MRT> in FP64"""
    f, _ = _states(np.zeros(19), 300, 11 + les, 0.01)
    g = f.copy()
    om, cs = 1 / 0.52, 0.01
    cellops.cell_collide_d(MRT, les, ctypes.c_double(om), ctypes.c_double(cs), ctypes.c_double(0.0), _ptr(f), len(f))
    cellops.cell_collide_mrt_dev_d(les, ctypes.c_double(om), ctypes.c_double(cs), ctypes.c_double(0.0), _ptr(g), len(g))
    np.testing.assert_allclose(g, f, rtol=0, atol=1e-11)


def test_moment_stress_equals_pi_neq(cellops):
    """Pi_neq taken from the collision's moments (the closure's features)
    equals sum c c f - rho/3 I - j j of the populations (pi_neq)"""
    f, _ = _states(np.zeros(19), 300, 5, 0.02)
    n = len(f)
    r1, r2 = np.zeros(n), np.zeros(n)
    p1, p2 = np.zeros((n, 6)), np.zeros((n, 6))
    cellops.cell_pi_neq_d(_ptr(f), _ptr(r1), _ptr(p1), n)
    cellops.cell_mrt_dev_pi_d(_ptr(f), _ptr(r2), _ptr(p2), n)
    np.testing.assert_allclose(r2, r1, rtol=1e-14)
    np.testing.assert_allclose(p2, p1, rtol=0, atol=1e-13)
