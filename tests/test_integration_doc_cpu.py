"""The C examples of INTEGRATION.md compile against include/lbm_gb300.h: the
whole program links against the built library (it is not run: no GPU is
needed), and each fragment compiles inside a function that declares its
free variables with the types a caller would hold.  A call whose argument
count or types drifted from the header fails here."""
from __future__ import annotations

import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

# free variables of the fragments, keyed by a name before the fragment's first call
DECLS = {
    "lbm_stream_collide_f32": """
        const float* fA = 0; float* fB = 0; const uint8_t* mask = 0;
        int nx = 64, ny = 24, nz = 6, pitch = 64, t = 0; float omega = 1.9f;
        const float UMAX = 0.05f; void* stream = 0; double* d_force3 = 0; double* d_scratch = 0;""",
    "lbm_force_stats": """
        const float* fxyz = 0; const double* fxyz_d = 0; int n = 10, t_start = 0, t_end = 10, nx = 8, ny = 8, nz = 4;
        double umax = 0.05, r = 4.0, nu = 1e-3; float u_tau = 0.01f;
        const float *v_mean = 0, *u_fl = 0, *v_fl = 0, *w_fl = 0, *stats4 = 0;
        float *yp = 0, *vp = 0, *ur = 0, *vr = 0, *wr = 0, *uave = 0, *urms = 0, *vave = 0, *vrms = 0;""",
    "lbm_save_state": """
        lbm_handle* h = 0;""",
    "float off[19]": """
        const lbm_handle* h = 0;""",
    "lbm_handle": """
        const char* text = "";""",
}


def _c_blocks():
    text = (ROOT / "INTEGRATION.md").read_text()
    return [b for lang, b in re.findall(r"```(\w*)\n(.*?)```", text, re.S) if lang == "c"]


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    return cc


def test_program_example_compiles_and_links(product, tmp_path):
    blocks = _c_blocks()
    main = next(b for b in blocks if "int main(" in b)
    src = tmp_path / "main.c"
    src.write_text(main)
    lib_dir = Path(product.__file__).parent / "_build"
    r = subprocess.run([_cc(), "-std=c11", "-Wall", "-Werror=implicit-function-declaration", str(src),
                        f"-I{ROOT / 'include'}", f"-L{lib_dir}", "-llbm_gb300", "-o", str(tmp_path / "main")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_fragments_compile(tmp_path):
    frags = [b for b in _c_blocks() if "int main(" not in b]
    assert len(frags) >= 4
    for i, frag in enumerate(frags):
        head = frag.split("(")[0]  # up to the fragment's first call
        key = next((k for k in DECLS if k in head), None)
        assert key is not None, frag
        src = tmp_path / f"frag{i}.c"
        src.write_text('#include <stdint.h>\n#include <stddef.h>\n#include "lbm_gb300.h"\n'
                       f"void fragment(void) {{\n{DECLS[key]}\n{frag}\n}}\n")
        r = subprocess.run([_cc(), "-std=c11", "-fsyntax-only", "-Werror=implicit-function-declaration",
                            "-Werror=incompatible-pointer-types", "-Werror=int-conversion", str(src),
                            f"-I{ROOT / 'include'}"], capture_output=True, text=True)
        assert r.returncode == 0, (frag, r.stderr)


def test_python_examples_use_the_package_api(product):
    """the Python examples parse, and every `lbm.X` and every method they
    call on a Solver (`s.`) or an Ensemble (`e.`) exists; every `lib.X` is a
    symbol the library exports"""
    import ast
    import ctypes

    text = (ROOT / "INTEGRATION.md").read_text()
    blocks = [b for lang, b in re.findall(r"```(\w*)\n(.*?)```", text, re.S) if lang == "python"]
    assert len(blocks) >= 3
    owners = {"lbm": product, "s": product.Solver, "e": product.Ensemble,
              "lib": ctypes.CDLL(str(Path(product.__file__).parent / "_build" / "liblbm_gb300.so"))}
    seen = 0
    for b in blocks:
        for node in ast.walk(ast.parse(b)):
            if isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name) and node.value.id in owners:
                assert hasattr(owners[node.value.id], node.attr), (node.value.id, node.attr)
                seen += 1
    assert seen >= 10
