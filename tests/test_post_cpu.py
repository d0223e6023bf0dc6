"""Post-processing against the reference's own programs, compiled from their
sources by oracle/ref_recipe.py (constants and file names adapted, see
POST_PROGRAMS there): ForceCalcs on a .force file, VelProf on a slice file.
Outputs are compared as the programs print them (6 significant digits).
Host only: no device is used."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import ref_recipe  # noqa: E402


def _ref_program(name: str) -> Path:
    p = ref_recipe.REF_DIR / name
    if not p.exists():
        if ref_recipe.staged() or ref_recipe.stage():
            ref_recipe.build_ref()
    if not p.exists():
        pytest.skip(f"reference program {name} not staged")
    return p


def _g(v: float) -> str:
    return f"{float(v):g}"


def test_force_stats_match_forcecalcs(product, tmp_path):
    lbm = product
    exe = _ref_program("forcecalcs")
    t = np.arange(300)
    rng = np.random.default_rng(3)
    fx = 1.52 + 0.04 * np.sin(2 * np.pi * t / 37) + 0.01 * rng.standard_normal(300)
    fy = 0.7 * np.sin(2 * np.pi * t / 74) + 0.02 * rng.standard_normal(300)
    fz = 1e-3 * rng.standard_normal(300)
    # the .force layout of WriteForces (LR7:2537-2545): "t, fx, fy, fz"
    lines = [f"{i}, {_g(a)}, {_g(b)}, {_g(c)}" for i, a, b, c in zip(t, fx, fy, fz)]
    (tmp_path / "post.force").write_text("\n".join(lines) + "\n")
    out = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=60).stdout.splitlines()
    vals = np.array([[float(x) for x in l.split(", ")[1:]] for l in lines], np.float32)
    mean, rms = lbm.force_stats(vals, 100, 300)
    want = [f"F{c}Av = {_g(m)}, F{c}RMS = {_g(r)}" for c, m, r in zip("xyz", mean, rms)]
    assert out == want


def test_wall_profile_matches_velprof(product, tmp_path):
    lbm = product
    exe = _ref_program("velprof")
    n = 32  # the program reads xDim / 2 = 32 lines
    rng = np.random.default_rng(4)
    vm = (0.05 * np.tanh(np.arange(n) / 6.0)).astype(np.float32)
    uf, vf, wf = (np.abs(rng.standard_normal((3, n))) * 1e-5).astype(np.float32)
    rows = ["VARIABLES = \"X\",\"Y\",\"Z\",...", "ZONE F=POINT"]
    for i in range(n):
        rows.append(", ".join([str(i), "0", "0", "0", "0", "0", "1", "0", _g(vm[i]), "0", _g(uf[i]), _g(vf[i]),
                               _g(wf[i])]))
    (tmp_path / "post_slice.dat").write_text("\n".join(rows) + "\n")
    subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=60, check=True)
    prof = (tmp_path / "post.prof").read_text().splitlines()
    assert prof[0] == "x,u,v,urms,vrms"
    parse = lambda s: np.float32(float(s))  # noqa: E731
    vmr = np.array([parse(_g(v)) for v in vm])
    ufr, vfr, wfr = (np.array([parse(_g(v)) for v in a]) for a in (uf, vf, wf))
    # the program's nu = uMax d / Re in FP32, and u_tau = 0.004 from row 1 on
    nu = np.float32(np.float32(0.06) * np.float32(62.0)) / np.float32(15000.0)
    got = lbm.wall_profile(vmr, ufr, vfr, wfr, 0.004, float(nu))
    for i in range(1, n):
        want = prof[1 + i]
        mine = ",".join([str(i)] + [_g(got[k, i]) for k in range(5)])
        assert mine == want, (i, mine, want)


def test_force_coefficients_of_a_known_signal(product):
    lbm = product
    t = np.arange(20000)
    u, d, lz = 0.05, 16.0, 128.0
    q = 0.5 * u * u * d * lz
    f = np.zeros((t.size, 3))
    f[:, 0] = 1.4 * q + 0.01 * q * np.sin(2 * np.pi * t / 400)
    f[:, 1] = 0.6 * q * np.sin(2 * np.pi * t * 0.00125 + 0.3)   # St = 0.00125 * 16 / 0.05 = 0.4
    c = lbm.force_coefficients(f, 4000, u, d, lz)
    assert abs(c["cd"] - 1.4) < 1e-3
    assert abs(c["cl_rms"] - 0.6 / np.sqrt(2)) < 5e-3
    assert abs(c["st"] - 0.4) < 2e-3


def test_stats_profiles_average_over_z(product):
    lbm = product
    rng = np.random.default_rng(5)
    s = rng.random((4, 6, 10, 12)).astype(np.float32)
    got = lbm.stats_profiles(s, 7)
    np.testing.assert_allclose(got, s[:, :, :, 7].mean(axis=1), rtol=1e-6)


def test_centerline_profiles_match_velplus(product, tmp_path):
    """velplus on a zone file of the reference's WriteResults layout (the
    writer here produces it), against lbm_centerline_profiles on the
    statistics as that file prints them"""
    lbm = product
    exe = _ref_program("velplus")
    nx, ny, nz, umax = 24, 24, 6, 0.06  # the staged program's xDim, yDim, zDim and uMax
    text = lbm.make_inputs(nx, ny, nz, geometry="periodic", umax=umax)
    rng = np.random.default_rng(11)
    f = (np.full((19, nz, ny, nx), 1 / 19) + 1e-3 * rng.standard_normal((19, nz, ny, nx))).astype(np.float32)
    st = np.stack([0.05 + 0.01 * rng.standard_normal((nz, ny, nx)), 0.01 * rng.standard_normal((nz, ny, nx)),
                   1e-5 * rng.random((nz, ny, nx)), 1e-5 * rng.random((nz, ny, nx))]).astype(np.float32)
    zone, _ = lbm.format_tecplot(text, f, 0, st)
    (tmp_path / "post.dat").write_text(zone)
    subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=60, check=True)
    out = (tmp_path / "post.vel").read_text().splitlines()
    assert out[0] == "x,u,v,urms,vrms" and len(out) == 1 + nx
    # the statistics as the zone file holds them
    rows = np.array([[float(t) for t in line.split(",")] for line in zone.splitlines()[2:]])
    printed = rows[:, 7:11].T.reshape(4, nz, ny, nx).astype(np.float32)
    got = lbm.centerline_profiles(printed, umax)
    for i in range(nx):
        mine = ",".join([_g(np.float32(i) / nx)] + [_g(got[k][i]) for k in ("uave", "vave", "urms", "vrms")])
        assert mine == out[1 + i], (i, mine, out[1 + i])
