"""Build liblbm_gb300.so in-tree (lbm_multigpu_gb300/_build/) with nvcc for sm_103a.

Translation units compiled in parallel and linked into one shared library:
the CUDA kernels (csrc/lbm_kernels.cu, and csrc/lbm_blocked.cu for the
blocked population layout), the C ABI host side
(csrc/lbm_host.cpp), the allocation-free force entry point
(csrc/lbm_noalloc.cu), and the learned subgrid closure (csrc/sgs_mlp.cu
kernels, csrc/lbm_sgs.cpp host side), and the ensemble of periodic boxes
(csrc/ensemble.cu, csrc/lbm_ensemble.cpp), and the post-processing of the
outputs (csrc/lbm_post.cpp).  Host code is built with -ffp-contract=off so geometry
masks and the text writers give identical results on x86 and aarch64 hosts.
Beside the library: the command lbm_run (csrc/lbm_run.cpp), the reference
programs' main() over the C ABI.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = PKG.parent / "include"
LIB = BUILD / "liblbm_gb300.so"
RUN = BUILD / "lbm_run"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[Path]:
    return [CSRC / "lbm_kernels.cu", CSRC / "lbm_blocked.cu", CSRC / "lbm_host.cpp", CSRC / "lbm_noalloc.cu", CSRC / "sgs_mlp.cu",
            CSRC / "lbm_sgs.cpp", CSRC / "ensemble.cu", CSRC / "lbm_ensemble.cpp", CSRC / "lbm_post.cpp"]


def _stale(out: Path, deps: list[Path]) -> bool:
    return not out.exists() or out.stat().st_mtime < max(d.stat().st_mtime for d in deps)


def build_run(force: bool = False) -> Path:
    """the lbm_run command, linked against the library next to it"""
    src = CSRC / "lbm_run.cpp"
    if not force and not _stale(RUN, [src, LIB, *sorted(INCLUDE.glob("*.h"))]):
        return RUN
    tmp = RUN.with_name(f"lbm_run.{os.getpid()}.tmp")
    r = subprocess.run([nvcc(), "-O2", "-std=c++17", f"-I{INCLUDE}", "-x", "c++", str(src), "-o", str(tmp),
                        f"-L{BUILD}", "-llbm_gb300", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"lbm_run build failed:\n{r.stdout}{r.stderr}")
    os.replace(tmp, RUN)
    return RUN


def build(force: bool = False, verbose: bool = False) -> Path:
    deps = sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    if not force and not _stale(LIB, deps):
        build_run()
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.name + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = [cc, *NVCC_FLAGS, "-x", "c++", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(len(sources())) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB.with_suffix(f".so.{os.getpid()}.tmp")
    r = subprocess.run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    build_run(force=True)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
