"""Build recipe for the checker side: the CPU oracle and the staged reference.

TEST INFRASTRUCTURE ONLY.  Nothing here is part of the product path.

* ``build_oracle()`` compiles this directory's CPU restatement
  (lbm_oracle.cpp, sgs_oracle.cpp) into ``oracle/_build/liblbm_oracle.so``.
* ``stage()`` reads the reference sources from ``$LBM_REFERENCE`` (the
  reference checkout; unset, nothing is staged) and
  writes copies of the code paths the tests need into ``oracle/_ref/``, which is
  git-ignored and travels to the GPU machine with the working tree:
    - ``lr7_body.inc``: LRTurbTest/LRMultiGPU7.cu from ImageFcnLR up to main()
      (device math, kernels, writers; LR7:68-2573);
    - ``di3_body.inc``: MRTtest/DynInlet3.cu device functions (DI3:62-1185);
    - ``cpu3d_body.inc``: CPU_3D/CPU_3D.cpp per-cell functions (CPU:116-1209);
    - ``cpu3d_<name>.cpp``: the CPU_3D program with its #define block set to a
      workload and the final output.dat dump switched off (timing only).
  The #define blocks of LR7 and DI3 are parsed into ``*_defines.json`` so the
  shims can be rebuilt for other configurations from the staged files alone.
* ``build_ref()`` compiles the host shims (ref_shim_*.cpp) against the staged
  code for each configuration in ``LR7_CONFIGS`` and the CPU_3D programs.

The reference is never built with its own build system and its sources are
never committed.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
BUILD_DIR = HERE / "_build"
# the reference checkout to stage from: $LBM_REFERENCE (unset: nothing is
# staged, and the copies already in _ref/, if any, are used)
REF_ROOT = Path(os.environ["LBM_REFERENCE"]) if os.environ.get("LBM_REFERENCE") else None

CXX = os.environ.get("CXX", "g++")
# identical FP32 arithmetic on x86 and aarch64 hosts: no contraction into FMA
ORACLE_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off"]
SHIM_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-w"]

# small configurations of the reference program used for parity fixtures
LR7_CONFIGS = {
    # MRT + Smagorinsky channel with a square body (the LR7 ImageFcn), no refinement
    "chan_les": dict(XDIM=64, YDIM=24, ZDIM=6, TMAX=200, STARTF=0, OBSTR1="4.f", OBSTX1="20.5f",
                     OBSTY1="11.5f", RE="60.f", UMAX="0.05f", SmagLES=1, CS="0.01f", REFINEMENT=0,
                     VELAV=1, START_VELAV=50, START_VELFLUC=120),
    # plain MRT (tau = 0.6), no refinement
    "chan_mrt": dict(XDIM=64, YDIM=24, ZDIM=6, TMAX=200, STARTF=0, OBSTR1="4.f", OBSTX1="20.5f",
                     OBSTY1="11.5f", RE="12.f", UMAX="0.05f", SmagLES=0, CS="0.01f", REFINEMENT=0,
                     VELAV=0, START_VELAV=100000, START_VELFLUC=250000),
    # two-level refinement: ratio-2 patch spanning the periodic z extent
    "lr": dict(XDIM=64, YDIM=24, ZDIM=4, TMAX=100, STARTF=0, OBSTR1="3.f", OBSTX1="20.5f",
               OBSTY1="11.5f", RE="60.f", UMAX="0.05f", SmagLES=1, CS="0.01f", REFINEMENT=1,
               LRFACTOR="0.5f", LRLEVEL=2, LRX0="12.25f", XLRDIM=32, LRY0="4.25f", YLRDIM=32,
               LRZ0="-0.75f", ZLRDIM=8, ORDER=2, BLOCKSIZELRX=32, VELAV=0, START_VELAV=100000, START_VELFLUC=250000),
    # refinement without LES
    "lr_mrt": dict(XDIM=64, YDIM=24, ZDIM=4, TMAX=100, STARTF=0, OBSTR1="3.f", OBSTX1="20.5f",
                   OBSTY1="11.5f", RE="20.f", UMAX="0.05f", SmagLES=0, CS="0.01f", REFINEMENT=1,
                   LRFACTOR="0.5f", LRLEVEL=2, LRX0="12.25f", XLRDIM=32, LRY0="4.25f", YLRDIM=32,
                   LRZ0="-0.75f", ZLRDIM=8, ORDER=2, BLOCKSIZELRX=32, VELAV=0, START_VELAV=100000, START_VELFLUC=250000),
    # the MRT + Smagorinsky channel over 1000 steps (the 1e-5 gate after 1000 steps)
    "chan_les_1k": dict(XDIM=64, YDIM=24, ZDIM=6, TMAX=1000, STARTF=0, OBSTR1="4.f", OBSTX1="20.5f",
                        OBSTY1="11.5f", RE="60.f", UMAX="0.05f", SmagLES=1, CS="0.01f", REFINEMENT=0,
                        VELAV=0, START_VELAV=100000, START_VELFLUC=250000),
    # the geometry of the 512x128x128 channel benchmark (square body of side 16
    # at x = 128): only its ImageFcn is evaluated (the mask fixture)
    "c2_geom": dict(XDIM=512, YDIM=128, ZDIM=128, TMAX=4, STARTF=0, OBSTR1="8.f", OBSTX1="128.5f",
                    OBSTY1="63.5f", RE="120.f", UMAX="0.05f", SmagLES=1, CS="0.01f", REFINEMENT=0,
                    VELAV=0, START_VELAV=100000, START_VELFLUC=250000),
    # tiny channel for the output-writer fixtures (statistics switch on at t = 5 and 12)
    "tiny": dict(XDIM=64, YDIM=8, ZDIM=4, TMAX=20, STARTF=0, OBSTR1="2.f", OBSTX1="20.5f", OBSTY1="3.5f",
                 RE="40.f", UMAX="0.05f", SmagLES=1, CS="0.01f", REFINEMENT=0, VELAV=1, START_VELAV=5,
                 START_VELFLUC=12),
}

# CPU_3D workloads: the baseline timing at the 512x128x128 channel shape and a
# small cavity (CPU_3D's own lid-driven cavity) for parity
CPU3D_PROGRAMS = {
    "c2": dict(XDIM=512, YDIM=128, ZDIM=128, TMAX=8),
    "c2_long": dict(XDIM=512, YDIM=128, ZDIM=128, TMAX=24),
    # its own lid-driven cavity, small, with the final output.dat kept (parity)
    "cav24": dict(XDIM=24, YDIM=24, ZDIM=24, TMAX=100),
    "cav24_1k": dict(XDIM=24, YDIM=24, ZDIM=24, TMAX=1000),
}
# programs whose output.dat is kept
CPU3D_KEEP_OUTPUT = {"cav24", "cav24_1k"}


# the reference's post-processing programs, staged with small constants
# (ForceCalcs reads lines tStart..tMax-1 of <casename>.force; VelProf reads
# xDim/2 lines of <casename>_slice.dat; its output loop runs to xDim over
# arrays of xDim/2 and is bounded to xDim/2 in the staged copy)
POST_PROGRAMS = {
    "forcecalcs": ("bgk_channel1/Re3000_Cyl2/ForceCalcs.cpp",
                   [(r"int tMax = \d+;", "int tMax = 300;"), (r"int tStart = \d+;", "int tStart = 100;"),
                    (r'string casename = "[^"]*";', 'string casename = "post";')]),
    "velprof": ("bgk_channel1/Re3000/VelProf.cpp",
                [(r'string casename = "[^"]*";', 'string casename = "post";'),
                 (r"for\(i = 0; i<xDim; i\+\+\)\{\n\toutput", "for(i = 0; i<xDim/2; i++){\n\toutput")]),
    "velplus": ("TurbChannel3/Re500/velplus.cpp",
                [(r"xDim = 128;", "xDim = 24;"), (r"yDim = 128;", "yDim = 24;"), (r"zDim = 16;", "zDim = 6;"),
                 (r'string casename = "[^"]*";', 'string casename = "post";')]),
}


def _cut(text: str, start_pat: str, stop_pat: str) -> str:
    lines = text.splitlines(keepends=True)
    i0 = next(i for i, l in enumerate(lines) if re.match(start_pat, l))
    i1 = next(i for i, l in enumerate(lines) if i > i0 and re.match(stop_pat, l))
    return "".join(lines[i0:i1])


def _parse_defines(text: str, stop_pat: str) -> dict:
    out = {}
    for line in text.splitlines():
        if re.match(stop_pat, line):
            break
        m = re.match(r"\s*#define\s+(\w+)\s+(.*)$", line)
        if not m:
            continue
        val = m.group(2).split("//")[0].strip().rstrip(";")
        out[m.group(1)] = val
    return out


def stage(ref_root: Path | None = REF_ROOT) -> bool:
    """Copy the needed reference code paths into oracle/_ref.  False if absent."""
    if ref_root is None:
        return False
    lr7 = ref_root / "LRTurbTest" / "LRMultiGPU7.cu"
    di3 = ref_root / "MRTtest" / "DynInlet3.cu"
    cpu = ref_root / "CPU_3D" / "CPU_3D.cpp"
    if not (lr7.exists() and di3.exists() and cpu.exists()):
        return False
    REF_DIR.mkdir(parents=True, exist_ok=True)
    t = lr7.read_text(errors="replace")
    (REF_DIR / "lr7_body.inc").write_text(_cut(t, r"inline __device__ int ImageFcnLR", r"int main\("))
    (REF_DIR / "lr7_defines.json").write_text(json.dumps(_parse_defines(t, r"inline __device__"), indent=1))
    t = di3.read_text(errors="replace")
    (REF_DIR / "di3_body.inc").write_text(_cut(t, r"inline __device__ int ImageFcnLR", r"__global__"))
    (REF_DIR / "di3_defines.json").write_text(json.dumps(_parse_defines(t, r"inline __device__"), indent=1))
    t = cpu.read_text(errors="replace")
    (REF_DIR / "cpu3d_body.inc").write_text(_cut(t, r"inline void bgk_collide", r"int main\(\)"))
    (REF_DIR / "cpu3d_defines.json").write_text(json.dumps(_parse_defines(t, r"inline int ImageFcn"), indent=1))
    for name, cfg in CPU3D_PROGRAMS.items():
        s = t
        for k, v in cfg.items():
            s = re.sub(rf"(#define\s+{k}\s+)\S+", rf"\g<1>{v}", s, count=1)
        if name not in CPU3D_KEEP_OUTPUT:
            # timing harness: the final tecplot dump of every node is not part of the loop
            s = s.replace('output.open ("output.dat");', "/* output.dat dump disabled for timing */")
        (REF_DIR / f"cpu3d_{name}.cpp").write_text(s)
    bc1 = ref_root / "BC1" / "LRMultiGPU7.cu"
    if bc1.exists():
        t = bc1.read_text(errors="replace")
        (REF_DIR / "bc1_westreg.inc").write_text(
            _cut(t, r"inline __device__ void West_Reg", r"(inline |__global__|__device__ |int main)"))
    for name, (rel, subs) in POST_PROGRAMS.items():
        src = ref_root / rel
        if not src.exists():
            continue
        s = src.read_text(errors="replace")
        for pat, rep in subs:
            s, n = re.subn(pat, rep, s, count=1)
            if n != 1:
                raise RuntimeError(f"staging {rel}: pattern {pat!r} not found")
        (REF_DIR / f"{name}.cpp").write_text(s)
    return True


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def oracle_lib_path() -> Path:
    return BUILD_DIR / "liblbm_oracle.so"


def build_oracle(force: bool = False) -> Path:
    out = oracle_lib_path()
    srcs = [HERE / "lbm_oracle.cpp", HERE / "sgs_oracle.cpp"]
    newest = max(p.stat().st_mtime for p in srcs + [HERE / "lbm_oracle.h"])
    if force or not out.exists() or out.stat().st_mtime < newest:
        BUILD_DIR.mkdir(parents=True, exist_ok=True)
        tmp = out.with_suffix(f".{os.getpid()}.tmp")
        _run([CXX, *ORACLE_FLAGS, "-o", str(tmp), *map(str, srcs)])
        os.replace(tmp, out)
    return out


def _dflags(defines: dict) -> list[str]:
    return [f"-D{k}={v}" for k, v in defines.items()]


def ref_lib_path(name: str) -> Path:
    return REF_DIR / f"lr7_{name}.so"


def staged() -> bool:
    return (REF_DIR / "lr7_body.inc").exists() and (REF_DIR / "lr7_defines.json").exists()


def build_ref(force: bool = False, jobs: int = 8) -> list[Path]:
    """Compile the shims against the staged reference code (needs stage())."""
    if not staged():
        return []
    base = json.loads((REF_DIR / "lr7_defines.json").read_text())
    jobs_list = []
    for name, cfg in LR7_CONFIGS.items():
        d = dict(base)
        d.update({k: str(v) for k, v in cfg.items()})
        out = ref_lib_path(name)
        if force or not out.exists():
            jobs_list.append([CXX, *SHIM_FLAGS, f"-I{REF_DIR}", *_dflags(d), "-o", str(out),
                              str(HERE / "ref_shim_lr7.cpp")])
    di3_defs = json.loads((REF_DIR / "di3_defines.json").read_text())
    di3_defs.pop("MODEL", None)
    out = REF_DIR / "di3.so"
    if force or not out.exists():
        jobs_list.append([CXX, *SHIM_FLAGS, f"-I{REF_DIR}", *_dflags(di3_defs), "-o", str(out),
                          str(HERE / "ref_shim_di3.cpp")])
    out = REF_DIR / "cpu3d.so"
    if force or not out.exists():
        cdefs = json.loads((REF_DIR / "cpu3d_defines.json").read_text())
        jobs_list.append([CXX, *SHIM_FLAGS, f"-I{REF_DIR}", *_dflags(cdefs), "-o", str(out),
                          str(HERE / "ref_shim_cpu3d.cpp")])
    for name in CPU3D_PROGRAMS:
        out = REF_DIR / f"cpu3d_{name}"
        if force or not out.exists():
            # portable flags: the same build on the x86 and the Arm host
            jobs_list.append([CXX, "-O3", "-w", "-o", str(out), str(REF_DIR / f"cpu3d_{name}.cpp")])
    out = REF_DIR / "bc1.so"
    if (REF_DIR / "bc1_westreg.inc").exists() and (force or not out.exists()):
        jobs_list.append([CXX, *SHIM_FLAGS, f"-I{REF_DIR}", "-o", str(out), str(HERE / "ref_shim_bc1.cpp")])
    for name in POST_PROGRAMS:
        src, out = REF_DIR / f"{name}.cpp", REF_DIR / name
        if src.exists() and (force or not out.exists()):
            jobs_list.append([CXX, "-O2", "-ffp-contract=off", "-w", "-o", str(out), str(src)])
    with ThreadPoolExecutor(jobs) as ex:
        list(ex.map(_run, jobs_list))
    return sorted(REF_DIR.glob("*.so"))


if __name__ == "__main__":
    ok = stage()
    print("staged reference:", ok)
    print("oracle:", build_oracle(force="--force" in sys.argv))
    for p in build_ref(force="--force" in sys.argv):
        print("ref:", p)
