"""Generate the golden fixtures of tests/golden/ from the reference's own code.

Runs the reference's device functions, kernels and writers (LRTurbTest/
LRMultiGPU7.cu, MRTtest/DynInlet3.cu, CPU_3D/CPU_3D.cpp) through the host
harness that oracle/ref_recipe.py stages and builds in oracle/_ref/ (needs the
reference sources, i.e. the development container).  Seeded inputs; rerunning
reproduces the files.

    python tests/golden/make_golden.py [part ...]   (all parts by default)
"""
from __future__ import annotations

import ctypes
import gzip
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import ref_recipe  # noqa: E402

P = ctypes.c_void_p
F = ctypes.c_float


def ptr(a):
    return a.ctypes.data_as(P)


def lib(name):
    return ctypes.CDLL(str(ref_recipe.REF_DIR / name))


CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 0, -1, 0, 0, 1, 0, -1, 0])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1, 0, 0, 1, 0, -1, 0, 0, 1, 0, -1])
CZ = np.array([0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1])
W = np.array([1 / 3] + [1 / 18] * 4 + [1 / 36] * 4 + [1 / 18] + [1 / 36] * 4 + [1 / 18] + [1 / 36] * 4)


def random_cells(n, seed):
    """near-equilibrium populations: BGK equilibrium of random (rho, j) plus noise"""
    rng = np.random.default_rng(seed)
    rho = 1 + 0.05 * rng.standard_normal(n)
    u = 0.06 * rng.standard_normal((3, n))
    cu = np.outer(CX, u[0]) + np.outer(CY, u[1]) + np.outer(CZ, u[2])
    feq = W[:, None] * (rho + 3 * cu + 4.5 * cu ** 2 - 1.5 * (u ** 2).sum(0))
    f = feq + 2e-3 * rng.standard_normal(feq.shape) * W[:, None]
    return np.ascontiguousarray(f.T, np.float32)


def fields(f):
    g = f.astype(np.float64)
    return np.stack([g.sum(0)] + [np.tensordot(c, g, 1) for c in (CX, CY, CZ)]).astype(np.float32)


def cells():
    n = 64
    f0 = random_cells(n, 20251203)
    out = dict(f0=f0)
    les = lib("lr7_chan_les.so")
    mrt = lib("lr7_chan_mrt.so")
    lr = lib("lr7_lr.so")
    di3 = lib("di3.so")
    c3 = lib("cpu3d.so")
    for om in (1.2, 1.8, 1.95):
        g = f0.copy()
        les.ref_mrt_collide(ptr(g), n, F(om))
        out[f"lr7_mrt_les_cs0.01_om{om}"] = g
        g = f0.copy()
        mrt.ref_mrt_collide(ptr(g), n, F(om))
        out[f"lr7_mrt_om{om}"] = g
        for use_mrt, name in ((1, "mrt"), (0, "bgk")):
            g = f0.copy()
            di3.ref_di3_collide(ptr(g), n, F(om), F(-5.16e-7), use_mrt)
            out[f"di3_{name}_les_cs0.02_dpdy-5.16e-7_om{om}"] = g
        g = f0.copy()
        c3.ref_cpu3d_mrt(ptr(g), n, F(om))
        out[f"cpu3d_mrt_om{om}"] = g
        g = f0.copy()
        c3.ref_cpu3d_bgk(ptr(g), n, F(om))
        out[f"cpu3d_bgk_om{om}"] = g
    for kind, val in ((3, 0.05), (4, 1.0), (5, 0.04), (6, 1.0)):
        g = f0.copy()
        les.ref_extrap(kind, ptr(g), n, F(val))
        out[f"extrap_{kind}_{val}"] = g
    g = f0.copy()
    c3.ref_cpu3d_lid_west(ptr(g), n)
    out["cpu3d_lid_west"] = g
    mom = np.zeros((n, 9), np.float32)
    les.ref_physical_moments(ptr(f0), ptr(mom), n)
    out["physical_moments"] = mom
    s = np.zeros((n, 6), np.float32)
    les.ref_strain_rate(ptr(mom), ptr(s), n)
    out["strain_rate"] = s
    for om in (1.9, 1.6):
        g = np.zeros((n, 19), np.float32)
        lr.ref_invert_les_cf(ptr(mom), ptr(g), n, F(om))
        out[f"invert_les_cf_cs0.01_lrf0.5_om{om}"] = g
        g = np.zeros((n, 19), np.float32)
        lr.ref_invert_les_fc(ptr(mom), ptr(g), n, F(om))
        out[f"invert_les_fc_cs0.01_lrf0.5_om{om}"] = g
    g = np.zeros(19, np.float32)
    les.ref_init_meq(ptr(g), F(0.05))
    out["init_meq_u0.05"] = g
    np.savez_compressed(HERE / "cells.npz", **out)


def write_inputs_text(L):
    buf = ctypes.create_string_buffer(1 << 14)
    n = L.ref_write_inputs(buf, len(buf))
    assert n > 0
    return buf.value.decode()


def runs(cases=(("chan_les", 200), ("chan_mrt", 200), ("lr", 100)), stem="runs"):
    meta = {}
    arrays = {}
    for name, steps in cases:
        cfg = ref_recipe.LR7_CONFIGS[name]
        L = lib(f"lr7_{name}.so")
        L.ref_setup(None, None)
        X, Y, Z = cfg["XDIM"], cfg["YDIM"], cfg["ZDIM"]
        img = np.zeros((Z, Y, X), np.int32)
        L.ref_image(ptr(img))
        arrays[f"{name}_image"] = img.astype(np.int16)
        L.ref_run(0, steps)
        f = np.zeros((19, Z, Y, X), np.float32)
        L.ref_get_coarse(ptr(f))
        arrays[f"{name}_fields"] = fields(f)
        Fr = np.zeros((3, cfg["TMAX"]), np.float32)
        L.ref_get_forces(ptr(Fr), cfg["TMAX"])
        arrays[f"{name}_forces"] = Fr[:, :steps].T.copy()
        prm = np.zeros(4, np.float32)
        L.ref_get_params(ptr(prm))
        arrays[f"{name}_params"] = prm
        meta[name] = dict(steps=steps, inputs=write_inputs_text(L), config={k: str(v) for k, v in cfg.items()})
        if cfg.get("REFINEMENT") == 1:
            fx, fy, fz = cfg["XLRDIM"], cfg["YLRDIM"], cfg["ZLRDIM"]
            ff = np.zeros((19, fz, fy, fx), np.float32)
            L.ref_get_fine(ptr(ff))
            arrays[f"{name}_fine_fields"] = fields(ff)
            imgf = np.zeros((fz, fy, fx), np.int32)
            L.ref_image_lr(ptr(imgf))
            arrays[f"{name}_fine_image"] = imgf.astype(np.int16)
    np.savez_compressed(HERE / f"{stem}.npz", **arrays)
    (HERE / f"{stem}.json").write_text(json.dumps(meta, indent=1))


def writer():
    """WriteInputs / WriteResults / WriteForces text of a tiny channel run"""
    cfg = ref_recipe.LR7_CONFIGS["tiny"]
    L = lib("lr7_tiny.so")
    L.ref_setup(None, None)
    steps = cfg["TMAX"]
    L.ref_run(0, steps)
    X, Y, Z = cfg["XDIM"], cfg["YDIM"], cfg["ZDIM"]
    f = np.zeros((19, Z, Y, X), np.float32)
    L.ref_get_coarse(ptr(f))
    zone = ctypes.create_string_buffer(1 << 22)
    sl = ctypes.create_string_buffer(1 << 20)
    assert L.ref_write_results(zone, len(zone), sl, len(sl)) == 0
    forces = ctypes.create_string_buffer(1 << 16)
    assert L.ref_write_forces(forces, len(forces), 0) > 0
    st = np.zeros((4, Z, Y, X), np.float32)
    L.ref_get_stats(ptr(st))
    Fr = np.zeros((3, steps), np.float32)
    L.ref_get_forces(ptr(Fr), steps)
    np.savez_compressed(HERE / "writer_tiny.npz", f=f, stats=st, forces=Fr.T.copy())
    for name, text in (("writer_tiny_part0.dat.gz", zone.value), ("writer_tiny_slice.dat.gz", sl.value)):
        with gzip.GzipFile(HERE / name, "wb", mtime=0) as fh:
            fh.write(text)
    (HERE / "writer_tiny.force").write_text(forces.value.decode())
    (HERE / "writer_tiny.inputs").write_text(write_inputs_text(L))


def cpu3d_cavity(name="cav24", steps=100, out="cpu3d_cavity24.npz"):
    """the reference CPU program's own lid-driven cavity (24^3, MRT with its
    quirks, `steps` steps): u, v, rho of its output.dat"""
    import os
    import subprocess
    import tempfile

    exe = ref_recipe.REF_DIR / f"cpu3d_{name}"
    with tempfile.TemporaryDirectory(dir=ref_recipe.REF_DIR) as d:
        r = subprocess.run([str(exe)], cwd=d, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        lines = open(os.path.join(d, "output.dat")).read().splitlines()[2:]
    n = 24
    uvrho = np.zeros((3, n, n, n), np.float32)
    for line in lines:
        x, y, z, u, v, w, rho = (float(t) for t in line.split(","))
        uvrho[:, int(z), int(y), int(x)] = (u, v, rho)
    np.savez_compressed(HERE / out, uvrho=uvrho, steps=steps)


def alt_bc():
    """the reference's alternate boundaries on seeded cells at every edge and
    corner class of their domains: CPU_3D's boundaries() dispatch (CPU:1027-
    1078) for the codes it routes (3 DirichletWest, 13 DirichletWest_Reg,
    14 NeumannEast_Reg, 54 NeumannEast_Regularized, 21/22 y symmetry, 23/24 z
    symmetry) on its YDIM x ZDIM face, its DirichletNorth_Reg / _South_Reg, LR7's xsymmetry_top / _bot on its own, and BC1's
    West_Reg at perturbed and plain time steps"""
    c3, lr7, bc1 = lib("cpu3d.so"), lib("lr7_tiny.so"), lib("bc1.so")
    out = {}

    def positions(ny, nz):
        ys = sorted({0, 1, ny // 2, ny - 2, ny - 1})
        zs = sorted({0, 1, nz // 2, nz - 2, nz - 1})
        return np.array([(y, z) for y in ys for z in zs], np.int32)

    ny, nz = c3.ref_cpu3d_ydim(), c3.ref_cpu3d_zdim()
    c3.ref_cpu3d_umax.restype = F
    yz = positions(ny, nz)
    f0 = random_cells(len(yz), 20251204)
    out.update(cpu3d_f0=f0, cpu3d_yz=yz, cpu3d_dims=np.array([ny, nz], np.int32),
               cpu3d_umax=np.float32(c3.ref_cpu3d_umax()))
    for im in (3, 13, 14, 54, 21, 22, 23, 24):
        g = f0.copy()
        c3.ref_cpu3d_boundary(ptr(g), len(yz), ptr(yz), im)
        out[f"cpu3d_im{im}"] = g
    for north in (1, 0):
        g = f0.copy()
        c3.ref_cpu3d_dirichlet_ns(ptr(g), len(yz), ptr(yz), north)
        out[f"cpu3d_dirichlet_north{north}"] = g
    ny, nz = lr7.ref_ydim(), lr7.ref_zdim()
    yz = positions(ny, nz)
    f0 = random_cells(len(yz), 20251205)
    out.update(lr7_f0=f0, lr7_yz=yz, lr7_dims=np.array([ny, nz], np.int32))
    for top in (1, 0):
        g = f0.copy()
        lr7.ref_xsymmetry(ptr(g), len(yz), ptr(yz), top)
        out[f"lr7_xsym_top{top}"] = g
    f0 = random_cells(32, 20251206)
    out["bc1_f0"] = f0
    for t in (1, 1000, 2000, 3000, 4000):
        g = f0.copy()
        bc1.ref_west_reg(ptr(g), len(g), F(0.05), t)
        out[f"bc1_west_reg_u0.05_t{t}"] = g
    np.savez_compressed(HERE / "alt_bc.npz", **out)


def masks():
    """the reference's ImageFcn (LR7:88-127) on the 512x128x128 channel
    benchmark's geometry (square body of side 16 at x = 128.5, y = 63.5),
    with the run record the reference writes for it"""
    cfg = ref_recipe.LR7_CONFIGS["c2_geom"]
    L = lib("lr7_c2_geom.so")
    X, Y, Z = cfg["XDIM"], cfg["YDIM"], cfg["ZDIM"]
    img = np.zeros((Z, Y, X), np.int32)
    L.ref_image(ptr(img))
    np.savez_compressed(HERE / "masks.npz", c2_image=img.astype(np.int16))
    (HERE / "masks.json").write_text(json.dumps(dict(c2=dict(inputs=write_inputs_text(L))), indent=1))


PARTS = dict(cells=lambda: cells(), runs=lambda: runs(), writer=lambda: writer(), masks=lambda: masks(),
             cpu3d_cavity=lambda: cpu3d_cavity(), alt_bc=lambda: alt_bc(),
             runs_1k=lambda: runs((("chan_les_1k", 1000),), "runs_1k"),
             cpu3d_cavity_1k=lambda: cpu3d_cavity("cav24_1k", 1000, "cpu3d_cavity24_1k.npz"))

if __name__ == "__main__":
    if not ref_recipe.staged():
        if not ref_recipe.stage():
            sys.exit("reference sources not found; set LBM_REFERENCE")
    ref_recipe.build_ref()
    for name in sys.argv[1:] or PARTS:
        PARTS[name]()
    for p in sorted(HERE.iterdir()):
        print(f"{p.stat().st_size:>9} {p.name}")
