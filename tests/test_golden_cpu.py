"""CPU tests: the oracle and the product's per-cell arithmetic against golden
vectors produced by the reference's own code (tests/golden/make_golden.py),
and the node masks against the reference's ImageFcn / ImageFcnLR, bit-exact.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np
import pytest

from oracle_bindings import REF_CODE, OracleRun, Refine, moments, ptr, rel_l2

ROOT = Path(__file__).resolve().parents[1]

F = ctypes.c_float
# FP32 per-cell tolerance: populations are O(0.05..0.33), the reference
# evaluates the same maps in another order
ATOL_CELL = 5e-7
# whole-run gate: velocity relative L2 after the run (1e-5 target)
RTOL_RUN = 1e-5


def _cells(golden):
    c = golden["cells"]
    return c, c["f0"].copy(), c["f0"].shape[0]


@pytest.mark.parametrize("om", [1.2, 1.8, 1.95])
def test_collide_oracle_and_product_vs_reference(golden, orc, cellops, om):
    c, f0, n = _cells(golden)
    cases = [
        # (fixture key, model id, les, cs, dpdy)
        (f"lr7_mrt_les_cs0.01_om{om}", 0, 1, 0.01, 0.0),
        (f"lr7_mrt_om{om}", 0, 0, 0.0, 0.0),
        (f"di3_mrt_les_cs0.02_dpdy-5.16e-7_om{om}", 1, 1, 0.02, -5.16e-7),
        (f"di3_bgk_les_cs0.02_dpdy-5.16e-7_om{om}", 2, 1, 0.02, -5.16e-7),
        (f"cpu3d_mrt_om{om}", 3, 0, 0.0, 0.0),
        (f"cpu3d_bgk_om{om}", 2, 0, 0.0, 0.0),
    ]
    for key, model, les, cs, dpdy in cases:
        want = c[key]
        g = f0.copy()
        orc.orc_collide(model, les, F(om), F(cs), F(dpdy), ptr(g), n)
        np.testing.assert_allclose(g, want, atol=ATOL_CELL, rtol=0, err_msg=f"oracle {key}")
        g = f0.copy()
        cellops.cell_collide(model, les, F(om), F(cs), F(dpdy), ptr(g), n)
        np.testing.assert_allclose(g, want, atol=ATOL_CELL, rtol=0, err_msg=f"product {key}")


@pytest.mark.parametrize("kind,val", [(3, 0.05), (4, 1.0), (5, 0.04), (6, 1.0)])
def test_extrap_vs_reference(golden, orc, cellops, kind, val):
    c, f0, n = _cells(golden)
    want = c[f"extrap_{kind}_{val}"]
    g = f0.copy()
    orc.orc_extrap(kind, ptr(g), n, F(val), F(val))
    np.testing.assert_allclose(g, want, atol=ATOL_CELL, rtol=0)
    g = f0.copy()
    cellops.cell_extrap(kind, ptr(g), n, F(val), F(val))
    np.testing.assert_allclose(g, want, atol=ATOL_CELL, rtol=0)


def test_moments_strain_and_rescale_vs_reference(golden, orc, cellops):
    c, f0, n = _cells(golden)
    for lib, fn in ((orc, "orc_physical_moments"), (cellops, "cell_physical_moments")):
        mom = np.zeros((n, 9), np.float32)
        getattr(lib, fn)(ptr(f0), ptr(mom), n)
        np.testing.assert_allclose(mom, c["physical_moments"], atol=1e-6, rtol=0)
    mom = c["physical_moments"].copy()
    for lib, fn in ((orc, "orc_strain_rate"), (cellops, "cell_strain_rate")):
        s = np.zeros((n, 6), np.float32)
        getattr(lib, fn)(ptr(mom), ptr(s), n)
        np.testing.assert_allclose(s, c["strain_rate"], atol=1e-9, rtol=1e-5)
    for om in (1.9, 1.6):
        g = np.zeros((n, 19), np.float32)
        orc.orc_invert_les_cf(ptr(mom), ptr(g), n, F(om), F(0.01), F(0.5))
        np.testing.assert_allclose(g, c[f"invert_les_cf_cs0.01_lrf0.5_om{om}"], atol=ATOL_CELL, rtol=0)
        g = np.zeros((n, 19), np.float32)
        orc.orc_invert_les_fc(ptr(mom), ptr(g), n, F(om), F(0.01), F(0.5))
        np.testing.assert_allclose(g, c[f"invert_les_fc_cs0.01_lrf0.5_om{om}"], atol=ATOL_CELL, rtol=0)


def test_init_equilibrium_vs_reference(golden, cellops):
    want = golden["cells"]["init_meq_u0.05"]
    mom = np.array([[1.0, 0.05, 0, 0, 0, 0, 0, 0, 0]], np.float32)
    g = np.zeros((1, 19), np.float32)
    cellops.cell_invert_scaled(ptr(mom), F(0.0), ptr(g), 1)
    np.testing.assert_allclose(g[0], want, atol=1e-8, rtol=0)


def _mask_codes(m):
    out = np.zeros(m.shape, np.int32)
    for k, v in REF_CODE.items():
        out[m == k] = v
    return out


@pytest.mark.parametrize("name", ["chan_les", "chan_mrt", "lr"])
def test_masks_bit_exact_vs_imagefcn(golden, product, orc, name):
    meta = golden["meta"][name]
    text = meta["inputs"]
    img = golden["runs"][f"{name}_image"]
    Z, Y, X = img.shape
    m = product.inputs_mask(text, 0).reshape(Z, Y, X)
    np.testing.assert_array_equal(_mask_codes(m), img)
    cfg = meta["config"]
    mo = np.zeros((Z, Y, X), np.uint8)
    orc.orc_mask_channel(ptr(mo), X, Y, Z, 1, F(float(cfg["OBSTX1"].rstrip("f"))), F(float(cfg["OBSTY1"].rstrip("f"))),
                         F(float(cfg["OBSTR1"].rstrip("f"))))
    np.testing.assert_array_equal(_mask_codes(mo), img)
    if f"{name}_fine_image" in golden["runs"]:
        fimg = golden["runs"][f"{name}_fine_image"]
        fm = product.inputs_mask(text, 1).reshape(fimg.shape)
        np.testing.assert_array_equal(_mask_codes(fm), fimg)


@pytest.mark.parametrize("name", ["chan_les", "chan_mrt", "lr"])
def test_relaxation_parameters_vs_reference(golden, product, name):
    """omega, omegaLR (LR7:2607-2617) recomputed from the record"""
    prm = golden["runs"][f"{name}_params"]
    text = golden["meta"][name]["inputs"]
    norm = product.normalize_inputs(text)
    assert norm == text
    got = {l.split("\t")[0].strip(): l.split("\t")[1] for l in norm.splitlines()}
    assert got["omega"] == ": " + f"{prm[0]:.6g}"
    assert got["omega in LR"] == ": " + f"{prm[1]:.6g}"


def _oracle_run(golden, name):
    meta = golden["meta"][name]
    cfg = meta["config"]
    prm = golden["runs"][f"{name}_params"]
    img = golden["runs"][f"{name}_image"]
    Z, Y, X = img.shape
    inv = {v: k for k, v in REF_CODE.items()}
    mask = np.vectorize(inv.get)(img).astype(np.uint8)
    les = int(cfg["SmagLES"])
    cs = float(cfg["CS"].rstrip("f"))
    refine = None
    if int(cfg["REFINEMENT"]) == 1:
        fimg = golden["runs"][f"{name}_fine_image"]
        fz, fy, fx = fimg.shape
        r = Refine(cnx=X, cny=Y, cnz=Z, fnx=fx, fny=fy, fnz=fz, lrx0=float(cfg["LRX0"].rstrip("f")),
                   lry0=float(cfg["LRY0"].rstrip("f")), lrz0=float(cfg["LRZ0"].rstrip("f")),
                   lrfactor=float(cfg["LRFACTOR"].rstrip("f")), lrlevel=int(cfg["LRLEVEL"]), order=int(cfg["ORDER"]),
                   cs=cs, omega_c=float(prm[0]), omega_f=float(prm[1]), quirk_fc_top_zflip=1)
        refine = dict(r=r, mask=np.vectorize(inv.get)(fimg).astype(np.uint8), omega_f=float(prm[1]))
    o = OracleRun(X, Y, Z, mask, float(prm[0]), model=0, les=les, cs=cs, u_in=float(cfg["UMAX"].rstrip("f")),
                  init_u=float(cfg["UMAX"].rstrip("f")), refine=refine)
    o.step(meta["steps"])
    return o, mask


@pytest.mark.parametrize("name", ["chan_les", "chan_mrt", "lr", "chan_les_1k"])
def test_oracle_whole_run_vs_reference_kernels(golden, name):
    """the oracle's restated time loop against the reference's own kernels
    (chan_les_1k: the MRT-LES channel over 1000 steps)"""
    o, mask = _oracle_run(golden, name)
    want = golden["runs"][f"{name}_fields"]
    fluid = (mask != 1) & (mask != 2)
    rho, j = moments(o.fa)
    assert rel_l2(j[:, fluid], want[1:, fluid]) < RTOL_RUN
    assert np.abs(rho[fluid] - want[0][fluid]).max() < 1e-5
    Fr = golden["runs"][f"{name}_forces"]
    Fo = np.array(o.forces)[: len(Fr)]
    assert rel_l2(Fo[:, 0], Fr[:, 0]) < 1e-5
    if f"{name}_fine_fields" in golden["runs"]:
        wf = golden["runs"][f"{name}_fine_fields"]
        fluid_f = o.fmask != 2
        _, jf = moments(o.ffa)
        assert rel_l2(jf[:, fluid_f], wf[1:, fluid_f]) < RTOL_RUN


def test_philox_noise_stream_bit_exact(orc, cellops):
    """product and oracle draw the same seeded inlet-noise numbers"""
    orc.orc_noise_uniform.restype = F
    for seed, cell, step in [(12345, 0, 0), (12345, 7, 3), (1, 2 ** 20, 999), (2 ** 31, 123456, 5000)]:
        a = orc.orc_noise_uniform(ctypes.c_uint32(seed), ctypes.c_uint32(cell), ctypes.c_uint32(step))
        b = cellops.cell_philox_uniform(ctypes.c_uint32(seed), ctypes.c_uint32(cell), ctypes.c_uint32(step))
        assert a == b and 0.0 <= a < 1.0
    xs = np.array([orc.orc_noise_uniform(ctypes.c_uint32(12345), ctypes.c_uint32(i), ctypes.c_uint32(1))
                   for i in range(4000)])
    assert abs(xs.mean() - 0.5) < 0.02 and abs(xs.var() - 1 / 12) < 0.01


def _cpu3d_cavity_inputs(product, n=24):
    return product.make_inputs(n, n, n, r1=5.0, re=50.0, umax=0.04, model="MRT_CPU3D", geometry="cavity",
                               lid_face="-x", lid_velocity=(0.0, 0.04, 0.0), init=2, init_velocity=0.04,
                               edge_pull="clamp", lid_bc="cpu3d")


@pytest.mark.parametrize("fixture", ["cpu3d_cavity24.npz", "cpu3d_cavity24_1k.npz"])
def test_oracle_vs_reference_cpu_program(golden, product, fixture):
    """the oracle in CPU_3D's semantics (clamped edge pulls, its regularised
    lid as written, its MRT, every node initialised at UMAX) against the
    output.dat of the reference CPU program itself (24^3 cavity, 100 and
    1000 steps)"""
    d = np.load(golden["dir"] / fixture)
    want, steps = d["uvrho"], int(d["steps"])
    n = 24
    mask = product.inputs_mask(_cpu3d_cavity_inputs(product)).reshape(n, n, n)
    assert (mask == 7).sum() == n * n and (mask[:, :, 0] == 7).all()
    omega = np.float32(1.0) / (np.float32(3.0) * (np.float32(0.04) * np.float32(10.0) / np.float32(50.0)) +
                               np.float32(0.5))
    o = OracleRun(n, n, n, mask, float(omega), model=3, init_kind=2, init_u=0.04, lid_u=(0, 0.04, 0), lid_face=0,
                  pull_clamp=1, lid_quirk=1)
    o.step(steps)
    rho, j = moments(o.fa)
    # the program prints 6 significant digits
    assert rel_l2(j[:2], want[:2]) < 1e-5
    assert np.abs(rho - want[2]).max() < 2e-5


def test_lid_regularisation_vs_reference(golden, orc, cellops):
    """CPU_3D's DirichletWest_Regularized, per cell"""
    c = golden["cells"]
    f0, want = c["f0"].copy(), c["cpu3d_lid_west"]
    n = f0.shape[0]
    for lib, fn in ((orc, "orc_lid"), (cellops, "cell_lid")):
        g = f0.copy()
        getattr(lib, fn)(ptr(g), n, 0, F(0.0), F(0.04), F(0.0), 1)
        np.testing.assert_allclose(g, want, atol=ATOL_CELL, rtol=0, err_msg=fn)


def test_c2_benchmark_mask_vs_imagefcn(product):
    """the mask of the 512x128x128 channel benchmark, from the record bench.py
    runs, equals the reference's ImageFcn (LR7:88-127) on that geometry node
    for node (tests/golden/masks.npz, made by make_golden.py)"""
    import json

    import bench

    img = np.load(ROOT / "tests" / "golden" / "masks.npz")["c2_image"]
    m = product.inputs_mask(bench.inputs_text("fp32", 10), 0).reshape(img.shape)
    np.testing.assert_array_equal(_mask_codes(m), img)
    text = json.loads((ROOT / "tests" / "golden" / "masks.json").read_text())["c2"]["inputs"]
    np.testing.assert_array_equal(_mask_codes(product.inputs_mask(text, 0).reshape(img.shape)), img)
    assert (img == 10).sum() == 16 * 16 * 128


def test_c3_circle_masks_vs_cylinder_rule(product):
    """the coarse and fine masks of the two-level refinement benchmark: the
    cylinder rule of CPU_3D's ImageFcn, (x - X)^2 + (y - Y)^2 < R^2 in FP32
    (CPU_3D/CPU_3D.cpp:41-42), on coarse nodes and on the fine nodes at
    LR location + i LR factor (ImageFcnLR's coordinates, LR7:68-86), with the
    channel's walls, inlet and outlet on the coarse level (LR7:88-127)"""
    import bench

    text = bench.c3_inputs(10)
    f32 = np.float32
    X, Y, R = f32(64.5), f32(63.5), f32(6.0)

    def circle(xc, yc):
        dx, dy = xc - X, yc - Y
        return (dx * dx + dy * dy) < R * R

    nx, ny, nz = 256, 128, 64
    m = product.inputs_mask(text, 0).reshape(nz, ny, nx)
    y, x = np.meshgrid(np.arange(ny, dtype=f32), np.arange(nx, dtype=f32), indexing="ij")
    want = np.where(circle(x, y), 2, 0).astype(np.uint8)
    want[:, 0], want[:, -1] = 3, 4
    want[0, :], want[-1, :] = 1, 1
    np.testing.assert_array_equal(m, np.broadcast_to(want, m.shape))
    fx, fy, fz = bench.C3_PATCH["lr_dims"]
    x0, y0, _ = (f32(v) for v in bench.C3_PATCH["lr_origin"])
    fm = product.inputs_mask(text, 1).reshape(fz, fy, fx)
    yy, xx = np.meshgrid(np.arange(fy, dtype=f32), np.arange(fx, dtype=f32), indexing="ij")
    fwant = np.where(circle(x0 + xx * f32(0.5), y0 + yy * f32(0.5)), 2, 0).astype(np.uint8)
    np.testing.assert_array_equal(fm, np.broadcast_to(fwant, fm.shape))
    assert (fwant == 2).sum() > 400  # the cylinder lies in the patch
