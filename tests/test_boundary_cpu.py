"""CPU tests of the drop-in boundary: the C-ABI library loads and exports
every symbol of include/lbm_gb300.h, the .inputs run records round-trip
byte-for-byte, and the tecplot/.force writers reproduce the reference's own
output (tests/golden/writer_tiny*) byte-for-byte.  No GPU needed."""
from __future__ import annotations

import gzip
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"


def _reference_root() -> Path:
    """the reference's sources as the oracle's recipe finds them (present only
    where the reference is checked out)"""
    import sys

    sys.path.insert(0, str(ROOT / "oracle"))
    import ref_recipe

    return ref_recipe.REF_ROOT


REFERENCE = _reference_root()


def header_symbols():
    text = (ROOT / "include" / "lbm_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*)\s+(lbm_\w+)\s*\(", text, re.M)))


def test_library_exports_every_header_symbol(product):
    lib = product.library()
    syms = header_symbols()
    assert len(syms) >= 25
    for name in syms:
        assert hasattr(lib, name), name
    bound = {n for n, _, _ in product.SIGNATURES}
    assert set(syms) <= bound, set(syms) - bound
    assert b"sm_103a" in lib.lbm_version()


def test_reference_run_records_round_trip(product):
    """every .inputs record of the reference parses and is written back
    identically, the derived omega / omegaLR lines recomputed"""
    files = sorted(REFERENCE.glob("**/*.inputs")) if REFERENCE and REFERENCE.exists() else []
    files += [GOLDEN / "writer_tiny.inputs"]
    for f in files:
        text = f.read_text()
        assert product.normalize_inputs(text) == text, f


def test_golden_records_round_trip(product, golden):
    for name, meta in golden["meta"].items():
        assert product.normalize_inputs(meta["inputs"]) == meta["inputs"], name


def test_tecplot_writer_byte_compatible(product):
    text = (GOLDEN / "writer_tiny.inputs").read_text()
    d = np.load(GOLDEN / "writer_tiny.npz")
    zone, slice_ = product.format_tecplot(text, d["f"], stats=d["stats"])
    assert zone == gzip.open(GOLDEN / "writer_tiny_part0.dat.gz", "rt").read()
    assert slice_ == gzip.open(GOLDEN / "writer_tiny_slice.dat.gz", "rt").read()


def test_force_writer_byte_compatible(product):
    text = (GOLDEN / "writer_tiny.inputs").read_text()
    d = np.load(GOLDEN / "writer_tiny.npz")
    assert product.format_forces(text, d["forces"].astype(np.float64)) == (GOLDEN / "writer_tiny.force").read_text()


def test_make_inputs_is_a_fixed_point(product):
    t = product.make_inputs(512, 128, 128, obst1=(128.5, 63.5, 0.0), r1=8.0, re=120.0, umax=0.05, les=1, cs=0.01,
                            geometry="channel_square", precision="fp16", inlet_noise=0.01, seed=12345)
    n = product.normalize_inputs(t)
    assert product.normalize_inputs(n) == n
    assert "omega \t: 1.92308" in n  # tau0 = 0.52
    t2 = product.make_inputs(64, 24, 6, geometry="channel_square", sgs="mlp", sgs_every=8)
    n2 = product.normalize_inputs(t2)
    assert "SGS every: \t8\n" in n2 and product.normalize_inputs(n2) == n2


@pytest.mark.parametrize("text,code,msg", [
    ("", 3, "no 'Base domain size'"),
    ("Base domain size 64x24x6\n", 3, "no TAB"),
    ("Base domain size \t64x24\n", 3, "cannot read"),
    ("Base domain size \t64x24x6\nRE: \tabc\n", 3, "cannot read"),
    ("Base domain size \t64x24x6\nWhat: \t1\n", 3, "unknown key"),
    ("Base domain size \t64x24x6\nSGS every: \t0\n", 3, "cannot read"),
    ("Base domain size \t64x24x6\nLAYOUT: \tweird\n", 3, "cannot read"),
    ("Base domain size \t64x24x6\nPRECISION: \tfp8\n", 3, "cannot read"),
])
def test_malformed_records_are_rejected(product, text, code, msg):
    with pytest.raises(product.LbmError) as e:
        product.normalize_inputs(text)
    assert e.value.code == code and msg in str(e.value)


@pytest.mark.parametrize("kw", [dict(geometry="dyninlet"), dict(geometry="channel_square", dpdy=-2e-6),
                                dict(geometry="cavity"), dict(geometry="channel_square", precision="fp64")])
def test_closure_configurations_are_rejected(product, kw):
    """the learned closure's collision carries no body force and runs on
    channel and periodic levels in FP32/FP16/BF16: other records are
    refused before any device work (LBM_ERR_CONFIG)"""
    t = product.make_inputs(64, 24, 6, obst1=(20.5, 11.5, 0.0), r1=4.0, re=60.0, umax=0.05, tmax=10, les=1,
                            sgs="mlp", **kw)
    with pytest.raises(product.LbmError) as e:
        product.Solver(t)
    assert e.value.code == 4 and "SGS mlp" in str(e.value)


def test_masks_of_every_geometry(product):
    for geom, expect in (("channel_square", {0, 1, 2, 3, 4}), ("channel_circle", {0, 1, 2, 3, 4}),
                         ("channel", {0, 1, 3, 4}), ("cavity", {0, 1, 7}), ("periodic", {0})):
        t = product.make_inputs(40, 20, 4, obst1=(15.5, 9.5, 0.0), r1=4.0, geometry=geom)
        m = product.inputs_mask(t).reshape(4, 20, 40)
        assert set(np.unique(m).tolist()) == expect, geom
    t = product.make_inputs(40, 20, 4, obst1=(15.5, 9.5, 0.0), r1=4.0, geometry="channel_circle")
    m = product.inputs_mask(t).reshape(4, 20, 40)
    y, x = np.mgrid[0:20, 0:40].astype(np.float32)
    circle = (x - np.float32(15.5)) ** 2 + (y - np.float32(9.5)) ** 2 < np.float32(16.0)
    inner = (x > 0) & (x < 39) & (y > 0) & (y < 19)
    assert np.array_equal((m[0] == 2) & inner, circle & inner)


def test_duct_and_faces_masks(product):
    """"duct" is CPU_3D's cylinder duct (CPU:39-63 with walls on the y and z
    faces, 3 = DirichletWest at x = 0, 14 = NeumannEast_Reg at x = nx-1);
    FACES puts a node type on each face with y faces over z over x"""
    N = product.NODE
    nx, ny, nz = 40, 20, 8
    t = product.make_inputs(nx, ny, nz, obst1=(15.5, 9.5, 0.0), r1=4.0, geometry="duct")
    m = product.inputs_mask(t).reshape(nz, ny, nx)
    z, y, x = np.mgrid[0:nz, 0:ny, 0:nx]
    want = np.zeros((nz, ny, nx), np.uint8)
    xf, yf = x.astype(np.float32), y.astype(np.float32)
    want[(xf - np.float32(15.5)) ** 2 + (yf - np.float32(9.5)) ** 2 < np.float32(16.0)] = N["BODY"]
    want[x == 0], want[x == nx - 1] = N["DIR_WEST"], N["NEU_EAST"]
    want[(z == 0) | (z == nz - 1)] = N["WALL"]
    want[(y == 0) | (y == ny - 1)] = N["WALL"]
    assert np.array_equal(m, want)
    faces = ("XSYM_BOT", "WEST_REG", "YSYM_BOT", "YSYM_TOP", "-", "ZSYM_TOP")
    t = product.make_inputs(nx, ny, nz, geometry="periodic", faces=faces)
    assert "FACES: \tXSYM_BOT WEST_REG YSYM_BOT YSYM_TOP - ZSYM_TOP" in product.normalize_inputs(t)
    m = product.inputs_mask(t).reshape(nz, ny, nx)
    want = np.zeros((nz, ny, nx), np.uint8)
    want[x == 0], want[x == nx - 1] = N["XSYM_BOT"], N["WEST_REG"]
    want[z == nz - 1] = N["ZSYM_TOP"]
    want[y == 0], want[y == ny - 1] = N["YSYM_BOT"], N["YSYM_TOP"]
    assert np.array_equal(m, want)
    for bad in ("DIR_WEST NEU_EAST", "DIR_WEST NEU_EAST - - - - -", "DIR_WEST X - - - -"):
        with pytest.raises(product.LbmError):
            product.inputs_mask(product.make_inputs(nx, ny, nz, faces=bad))


def test_checkpoint_rejects_other_files(product, tmp_path):
    """lbm_create_from_state reads the file's header before any device work"""
    import ctypes

    lib = product.library()
    bad = tmp_path / "x.ckpt"
    bad.write_bytes(b"not a checkpoint at all")
    h = ctypes.c_void_p()
    assert lib.lbm_create_from_state(str(bad).encode(), ctypes.byref(h)) == 3
    assert b"not a checkpoint" in lib.lbm_last_error()
    assert lib.lbm_create_from_state(str(tmp_path / "missing").encode(), ctypes.byref(h)) == 1


def test_lbm_run_command_arguments(product, tmp_path):
    """lbm_run (the reference programs' main() as a command) reports usage
    and unreadable records before any device work"""
    import subprocess

    from lbm_multigpu_gb300 import build

    exe = build.build_run()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage: lbm_run" in r.stderr
    r = subprocess.run([str(exe), "case.inputs", "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    r = subprocess.run([str(exe), str(tmp_path / "missing.inputs")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot read" in r.stderr
