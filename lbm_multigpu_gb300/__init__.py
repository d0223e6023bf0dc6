"""GB300-native D3Q19 lattice-Boltzmann stream-collide engine.

Python mirror of the C ABI in ``include/lbm_gb300.h`` (ctypes, no torch on the
hot path).  The compute path is ``lbm_multigpu_gb300/_build/liblbm_gb300.so``,
hand-written CUDA for sm_103a; importing this package never falls back to a
CPU implementation: if the library is missing, :func:`library` raises.

The reference (gladyslol/LBM_MultiGPU) is driven by ``#define`` blocks and
records each run in a ``.inputs`` file (LRTurbTest/LRMultiGPU7.cu:2547-2573);
:class:`Solver` takes that record as its configuration, and
:func:`make_inputs` writes one from keyword arguments.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

__all__ = ["Solver", "LbmError", "library", "make_inputs", "normalize_inputs", "inputs_mask", "format_tecplot", "format_forces", "NODE", "MODELS"]

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "liblbm_gb300.so"

NODE = dict(FLUID=0, WALL=1, BODY=2, WEST_INLET=3, EAST_OUTLET=4, SOUTH_INLET=5, NORTH_OUTLET=6, LID=7,
            DIR_WEST=8, NEU_EAST=9, NEU_EAST_REG=10, XSYM_TOP=11, XSYM_BOT=12, YSYM_TOP=13, YSYM_BOT=14,
            ZSYM_TOP=15, ZSYM_BOT=16, WEST_REG=17, DIR_WEST_V=18, DIR_NORTH=19, DIR_SOUTH=20)
MODELS = dict(MRT=0, MRT_DI3=1, BGK=2, MRT_CPU3D=3)

_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_SZ = ctypes.c_size_t

# (name, restype, argtypes) for every function of include/lbm_gb300.h
SIGNATURES = [
    ("lbm_last_error", ctypes.c_char_p, []),
    ("lbm_version", ctypes.c_char_p, []),
    ("lbm_inputs_normalize", _I, [ctypes.c_char_p, ctypes.c_char_p, _SZ, ctypes.POINTER(_SZ)]),
    ("lbm_inputs_mask", _I, [ctypes.c_char_p, _I, _P, _SZ, ctypes.POINTER(_SZ)]),
    ("lbm_format_tecplot", _I, [ctypes.c_char_p, _I, _P, _P, ctypes.c_char_p, _SZ, ctypes.POINTER(_SZ),
                                ctypes.c_char_p, _SZ, ctypes.POINTER(_SZ)]),
    ("lbm_format_forces", _I, [ctypes.c_char_p, _P, _I, ctypes.c_char_p, _SZ, ctypes.POINTER(_SZ)]),
    ("lbm_create", _I, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    ("lbm_destroy", _I, [_P]),
    ("lbm_get_dims", _I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    ("lbm_get_nlevels", _I, [_P, ctypes.POINTER(_I)]),
    ("lbm_get_params", _I, [_P, _P]),
    ("lbm_get_storage_offsets", _I, [_P, _I, _P]),
    ("lbm_get_time", _I, [_P, ctypes.POINTER(_I)]),
    ("lbm_get_mask", _I, [_P, _I, _P]),
    ("lbm_set_mask", _I, [_P, _I, _P]),
    ("lbm_init_equilibrium", _I, [_P]),
    ("lbm_get_populations", _I, [_P, _I, _P]),
    ("lbm_set_populations", _I, [_P, _I, _P]),
    ("lbm_step", _I, [_P, _I]),
    ("lbm_step_timed", _I, [_P, _I, ctypes.POINTER(_F)]),
    ("lbm_synchronize", _I, [_P]),
    ("lbm_get_fields", _I, [_P, _I, _P, _P, _P, _P]),
    ("lbm_get_stats", _I, [_P, _I, _P]),
    ("lbm_get_forces", _I, [_P, _P, _I, ctypes.POINTER(_I)]),
    ("lbm_get_last_force", _I, [_P, _P]),
    ("lbm_get_last_force_async", _I, [_P, _P]),
    ("lbm_mlp_param_count", _I, []),
    ("lbm_mlp_blob_bytes", _SZ, []),
    ("lbm_mlp_make_blob", _I, [_P, _P]),
    ("lbm_mlp_init_params", _I, [ctypes.c_uint32, _P]),
    ("lbm_mlp_grad", _I, [_P, _P, _P, _I, _P, _P, _P]),
    ("lbm_mlp_predict", _I, [_P, _P, _I, _P, _P]),
    ("lbm_mlp_train", _I, [_P, _P, _I, _I, _I, _F, ctypes.c_uint32, _P, _P, _P]),
    ("lbm_tc_selftest", _I, [_I, _P, _P, _P]),
    ("lbm_mlp_predict_tc", _I, [_P, _P, _I, _P, _P]),
    ("lbm_set_sgs_mlp", _I, [_P, _P, _I]),
    ("lbm_save_state", _I, [_P, ctypes.c_char_p]),
    ("lbm_get_dyn_history", _I, [_P, _P, _I, _P]),
    ("lbm_restore_state", _I, [_P, ctypes.c_char_p]),
    ("lbm_create_from_state", _I, [ctypes.c_char_p, _P]),
    ("lbm_force_stats", _I, [_P, _I, _I, _I, _P, _P]),
    ("lbm_force_coefficients", _I, [_P, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    _P, _P, _P]),
    ("lbm_wall_profile", _I, [_P, _P, _P, _P, _I, _F, _F, _P, _P, _P, _P, _P]),
    ("lbm_stats_profiles", _I, [_P, _I, _I, _I, _I, _P]),
    ("lbm_set_geometry", _I, [_P, _P]),
    ("lbm_write_tecplot", _I, [_P, ctypes.c_char_p]),
    ("lbm_centerline_profiles", _I, [_P, _I, _I, _I, ctypes.c_double, _P, _P, _P, _P]),
    ("lbm_ensemble_create", _I, [_I, _P, _P, _I, _F, _P]),
    ("lbm_ensemble_destroy", _I, [_P]),
    ("lbm_ensemble_init_turbulence", _I, [_P, ctypes.c_uint32, _F, _I, _I]),
    ("lbm_ensemble_modes", _I, [_P, _I, _P, _P, _P, _I, _P]),
    ("lbm_ensemble_init_filtered", _I, [_P, _P]),
    ("lbm_ensemble_set_mlp", _I, [_P, _P]),
    ("lbm_ensemble_autotune", _I, [_P, _P, _P, _P]),
    ("lbm_ensemble_step", _I, [_P, _I]),
    ("lbm_ensemble_step_timed", _I, [_P, _I, _P]),
    ("lbm_ensemble_info", _I, [_P, _P, _P, _P, _P]),
    ("lbm_ensemble_energy", _I, [_P, _P]),
    ("lbm_ensemble_velocity", _I, [_P, _I, _P]),
    ("lbm_ensemble_populations", _I, [_P, _I, _P]),
    ("lbm_ensemble_set_populations", _I, [_P, _I, _P]),
    ("lbm_ensemble_samples", _I, [_P, _F, _P, _P, ctypes.c_longlong, _P]),
    ("lbm_get_launch_count", _I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    ("lbm_time_stream_collide", _I, [_P, _I, _I, ctypes.POINTER(_F)]),
    ("lbm_audit", _I, [_P, _I, _P]),
    ("lbm_write_inputs", _I, [_P, ctypes.c_char_p, _SZ, ctypes.POINTER(_SZ)]),
    ("lbm_write_outputs", _I, [_P, ctypes.c_char_p]),
    ("lbm_stream_collide_f32", _I, [_P, _P, _P, _I, _I, _I, _I, _I, _I, _F, _F, _F, _F, _I, _P]),
    ("lbm_body_force_f32", _I, [_P, _P, _I, _I, _I, _I, _P, _P, _P]),
    ("lbm_body_force_scratch_doubles", _SZ, []),
    ("lbm_body_force_f32_noalloc", _I, [_P, _P, _I, _I, _I, _I, _P, _P]),
]


class LbmError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"lbm error {code}: {msg}")
        self.code = code


_lib = None


def library(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Load liblbm_gb300.so (built in-tree by lbm_multigpu_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run `python -m lbm_multigpu_gb300.build` (or __graft_entry__.build())")
    lib = ctypes.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        raise LbmError(rc, library().lbm_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return a.ctypes.data_as(_P)


def _fmt(v) -> str:
    # C++ ostream default formatting (6 significant digits) as WriteInputs uses
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    s = f"{float(np.float32(v)):.6g}"
    if "e" in s:
        m, e = s.split("e")
        s = f"{m}e{int(e):+03d}"
    return s


def make_inputs(nx: int, ny: int, nz: int, *, obst1=(0.0, 0.0, 0.0), r1=1.0, obst2=(0.0, 0.0, 0.0), r2=0.0,
                re=100.0, umax=0.05, tmax=1000, startf=0, start_velav=100000, start_velfluc=250000,
                refinement=0, model="MRT", les=0, cs=0.02, lr_dims=(128, 80, 8), lr_factor=0.5,
                lr_origin=(128.25, 64.25, -0.75), dpdy=None, **ext) -> str:
    """A .inputs record in the reference's WriteInputs layout (LR7:2547-2573).

    The derived ``omega`` lines are left for the library to recompute; extension
    keys (geometry, precision, tau, lid, noise, ...) are passed as keyword
    arguments named after the record keys: geometry="cavity", tau=0.6,
    lid_velocity=(0.05, 0, 0), lid_face="+z", precision="fp16",
    inlet_noise=0.01, seed=12345, velav=1, init=1, init_velocity=0.0,
    layout="blocked" (population layout: "soa", "blocked" or "auto"),
    faces=("DIR_WEST", "NEU_EAST", "YSYM_BOT", "YSYM_TOP", "-", "-") (a node
    type name from NODE per face x = 0, x = nx-1, y = 0, y = ny-1, z = 0,
    z = nz-1; "-" keeps the geometry's own).
    """
    def tup(t):
        return "(" + ",".join(_fmt(v) for v in t) + ")"

    lines = [
        ("Base domain size", f"{nx}x{ny}x{nz}"),
        ("Base blocksize:", "64x1x1"),
        ("Obst1 location:", tup(obst1)),
        ("Obst1 radius:", _fmt(r1)),
        ("Obst2 location:", tup(obst2)),
        ("Obst2 radius:", _fmt(r2)),
        ("RE:", _fmt(re)),
        ("UMAX:", _fmt(umax)),
        ("omega", ": 0"),  # derived; the library writes the value it computes
    ]
    if dpdy is not None:
        lines.append(("DPDY", ": " + _fmt(dpdy)))
    lines += [
        ("TMAX:", _fmt(tmax)),
        ("STARTF:", _fmt(startf)),
        ("START_VELAV:", _fmt(start_velav)),
        ("START_VELFLUC:", _fmt(start_velfluc)),
        ("REFINEMENT:", _fmt(refinement)),
        ("MODEL:", model),
        ("Smagorinsky LES:", _fmt(les)),
        ("CS:", _fmt(cs)),
        ("LR domain size", "x".join(str(int(v)) for v in lr_dims)),
        ("LR factor", _fmt(lr_factor)),
        ("LR location", "x".join(_fmt(v) for v in lr_origin)),
        ("LR blocksize:", "64x1x1"),
        ("omega in LR", ": 0"),
        ("GPUs per node", ": 1"),
    ]
    names = {"geometry": "GEOMETRY:", "precision": "PRECISION:", "tau": "TAU:", "lid_velocity": "LID velocity:",
             "lid_face": "LID face:", "inlet_noise": "Inlet noise:", "seed": "Seed:", "velav": "VELAV:",
             "init": "Init:", "init_velocity": "Init velocity:", "order": "ORDER:", "fc_top_zflip": "FC top zflip:",
             "edge_pull": "EDGE PULL:", "lid_bc": "LID BC:", "bounceback": "BOUNCEBACK:", "sgs": "SGS:",
             "sgs_weights": "SGS weights:", "sgs_every": "SGS every:", "dyny1": "DYNY1:", "dyn_every": "DYN every:",
             "dyn_start": "DYN start:", "trip_end": "TRIP end:", "kp": "KP:", "faces": "FACES:",
             "cf_time": "CF TIME:", "layout": "LAYOUT:"}
    for k, v in ext.items():
        if k not in names:
            raise KeyError(f"unknown .inputs extension key {k!r}")
        if k == "faces" and isinstance(v, (tuple, list)):
            v = " ".join(v)
        lines.append((names[k], tup(v) if isinstance(v, (tuple, list)) else (v if isinstance(v, str) else _fmt(v))))
    return "".join(f"{k} \t{v}\n" for k, v in lines)


def normalize_inputs(text: str) -> str:
    """Parse a record and write it back in the reference's format (no GPU)."""
    lib = library()
    n = _SZ(0)
    _check(lib.lbm_inputs_normalize(text.encode(), None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(lib.lbm_inputs_normalize(text.encode(), buf, n.value + 1, ctypes.byref(n)))
    return buf.value.decode()


def inputs_mask(text: str, level: int = 0) -> np.ndarray:
    """Node mask a record describes, uint8[nz][ny][nx] (no GPU)."""
    lib = library()
    n = _SZ(0)
    _check(lib.lbm_inputs_mask(text.encode(), level, None, 0, ctypes.byref(n)))
    m = np.zeros(n.value, np.uint8)
    _check(lib.lbm_inputs_mask(text.encode(), level, _ptr(m), m.size, ctypes.byref(n)))
    return m


def format_tecplot(text: str, f: np.ndarray, level: int = 0, stats: np.ndarray | None = None) -> tuple[str, str]:
    """(zone, slice) tecplot text of populations f in WriteResults' layout (no GPU)."""
    lib = library()
    f = np.ascontiguousarray(f, np.float32)
    st = None if stats is None else np.ascontiguousarray(stats, np.float32)
    n, m = _SZ(0), _SZ(0)
    args = (text.encode(), level, _ptr(f), None if st is None else _ptr(st))
    _check(lib.lbm_format_tecplot(*args, None, 0, ctypes.byref(n), None, 0, ctypes.byref(m)))
    a, b = ctypes.create_string_buffer(n.value + 1), ctypes.create_string_buffer(m.value + 1)
    _check(lib.lbm_format_tecplot(*args, a, n.value + 1, ctypes.byref(n), b, m.value + 1, ctypes.byref(m)))
    return a.value.decode(), b.value.decode()


def format_forces(text: str, forces: np.ndarray) -> str:
    """.force file text of a per-step force history (n, 3) (no GPU)"""
    lib = library()
    F = np.ascontiguousarray(forces, np.float64).reshape(-1, 3)
    n = _SZ(0)
    _check(lib.lbm_format_forces(text.encode(), _ptr(F), F.shape[0], None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(lib.lbm_format_forces(text.encode(), _ptr(F), F.shape[0], buf, n.value + 1, ctypes.byref(n)))
    return buf.value.decode()


class Solver:
    """One simulation on the current CUDA device (``lbm_create`` ... ``lbm_destroy``)."""

    def __init__(self, inputs_text: str):
        self._lib = library()
        h = _P()
        _check(self._lib.lbm_create(inputs_text.encode(), ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- shape and parameters --
    @property
    def nlevels(self) -> int:
        n = _I()
        _check(self._lib.lbm_get_nlevels(self._h, ctypes.byref(n)))
        return n.value

    def dims(self, level: int = 0) -> tuple[int, int, int]:
        a, b, c = _I(), _I(), _I()
        _check(self._lib.lbm_get_dims(self._h, level, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def params(self) -> dict:
        o = np.zeros(4, np.float32)
        _check(self._lib.lbm_get_params(self._h, _ptr(o)))
        return dict(omega=float(o[0]), omega_lr=float(o[1]), sf_cf=float(o[2]), sf_fc=float(o[3]))

    def storage_offsets(self, level: int = 0) -> np.ndarray:
        """the offsets FP16 / BF16 storage subtracts (zeros for FP32 / FP64)"""
        o = np.zeros(19, np.float32)
        _check(self._lib.lbm_get_storage_offsets(self._h, level, _ptr(o)))
        return o

    @property
    def time(self) -> int:
        t = _I()
        _check(self._lib.lbm_get_time(self._h, ctypes.byref(t)))
        return t.value

    # -- state --
    def mask(self, level: int = 0) -> np.ndarray:
        nx, ny, nz = self.dims(level)
        m = np.zeros((nz, ny, nx), np.uint8)
        _check(self._lib.lbm_get_mask(self._h, level, _ptr(m)))
        return m

    def set_mask(self, mask: np.ndarray, level: int = 0) -> None:
        nx, ny, nz = self.dims(level)
        m = np.ascontiguousarray(mask, np.uint8).reshape(nz, ny, nx)
        _check(self._lib.lbm_set_mask(self._h, level, _ptr(m)))

    def init_equilibrium(self) -> None:
        _check(self._lib.lbm_init_equilibrium(self._h))

    def populations(self, level: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        """populations float32[19][nz][ny][nx]; with out (C-contiguous
        float32 of that shape, e.g. pinned host memory) the copy lands there
        directly"""
        nx, ny, nz = self.dims(level)
        if out is None:
            f = np.empty((19, nz, ny, nx), np.float32)
        else:
            f = out
            if f.dtype != np.float32 or f.shape != (19, nz, ny, nx) or not f.flags["C_CONTIGUOUS"]:
                raise ValueError(f"out must be C-contiguous float32 of shape {(19, nz, ny, nx)}")
        _check(self._lib.lbm_get_populations(self._h, level, _ptr(f)))
        return f

    def set_populations(self, f: np.ndarray, level: int = 0) -> None:
        nx, ny, nz = self.dims(level)
        g = np.ascontiguousarray(f, np.float32).reshape(19, nz, ny, nx)
        _check(self._lib.lbm_set_populations(self._h, level, _ptr(g)))

    # -- time stepping --
    def step(self, n: int = 1) -> None:
        _check(self._lib.lbm_step(self._h, n))

    def step_timed(self, n: int) -> float:
        ms = _F()
        _check(self._lib.lbm_step_timed(self._h, n, ctypes.byref(ms)))
        return float(ms.value)

    def synchronize(self) -> None:
        _check(self._lib.lbm_synchronize(self._h))

    # -- outputs --
    def fields(self, level: int = 0) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
        nx, ny, nz = self.dims(level)
        out = [np.zeros((nz, ny, nx), np.float32) for _ in range(4)]
        _check(self._lib.lbm_get_fields(self._h, level, *(_ptr(a) for a in out)))
        return tuple(out)

    def stats(self, level: int = 0) -> np.ndarray:
        nx, ny, nz = self.dims(level)
        s = np.zeros((4, nz, ny, nx), np.float32)
        _check(self._lib.lbm_get_stats(self._h, level, _ptr(s)))
        return s

    def forces(self, max_steps: int | None = None) -> np.ndarray:
        n = max(self.time, 1) if max_steps is None else max_steps
        f = np.zeros((n, 3), np.float64)
        got = _I()
        _check(self._lib.lbm_get_forces(self._h, _ptr(f), n, ctypes.byref(got)))
        return f[: got.value]

    def last_force(self) -> np.ndarray:
        f = np.zeros(3, np.float64)
        _check(self._lib.lbm_get_last_force(self._h, _ptr(f)))
        return f

    def last_force_async(self, out: np.ndarray) -> None:
        """queue the copy of the last step's force into out (3 float64,
        ideally pinned); valid after synchronize()"""
        if out.dtype != np.float64 or out.size < 3 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float64 array of 3")
        _check(self._lib.lbm_get_last_force_async(self._h, _ptr(out)))

    def dyn_history(self) -> np.ndarray:
        """the dynamic inlet's control history, rows (t, mean v, dpdy)"""
        n = _I()
        _check(self._lib.lbm_get_dyn_history(self._h, None, 0, ctypes.byref(n)))
        h = np.zeros((n.value, 3), np.float32)
        if n.value:
            _check(self._lib.lbm_get_dyn_history(self._h, _ptr(h), n.value, ctypes.byref(n)))
        return h

    def save_state(self, path: str) -> None:
        """checkpoint: record, time, stored populations, statistics, forces"""
        _check(self._lib.lbm_save_state(self._h, str(path).encode()))

    def restore_state(self, path: str) -> None:
        _check(self._lib.lbm_restore_state(self._h, str(path).encode()))

    @classmethod
    def from_state(cls, path: str) -> "Solver":
        """a solver made from the record inside a checkpoint, at its state"""
        self = cls.__new__(cls)
        self._lib = library()
        h = _P()
        _check(self._lib.lbm_create_from_state(str(path).encode(), ctypes.byref(h)))
        self._h = h
        return self

    def set_sgs_mlp(self, params: np.ndarray) -> None:
        """weights of the learned closure (the record must select sgs="mlp")"""
        p = np.ascontiguousarray(params, np.float32)
        _check(self._lib.lbm_set_sgs_mlp(self._h, _ptr(p), p.size))

    def launch_count(self) -> int:
        """kernels launched by this solver so far"""
        n = ctypes.c_longlong()
        _check(self._lib.lbm_get_launch_count(self._h, ctypes.byref(n)))
        return int(n.value)

    def time_stream_collide(self, n: int, level: int = 0) -> float:
        ms = _F()
        _check(self._lib.lbm_time_stream_collide(self._h, level, n, ctypes.byref(ms)))
        return float(ms.value)

    def audit(self, level: int = 0) -> np.ndarray:
        o = np.zeros(4, np.float64)
        _check(self._lib.lbm_audit(self._h, level, _ptr(o)))
        return o

    def inputs_text(self) -> str:
        n = _SZ(0)
        _check(self._lib.lbm_write_inputs(self._h, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value + 1)
        _check(self._lib.lbm_write_inputs(self._h, buf, n.value + 1, ctypes.byref(n)))
        return buf.value.decode()

    def write_outputs(self, casename: str) -> None:
        _check(self._lib.lbm_write_outputs(self._h, casename.encode()))

    def write_tecplot(self, casename: str) -> None:
        """CASENAME_part<n>.dat and CASENAME_slice.dat only"""
        _check(self._lib.lbm_write_tecplot(self._h, casename.encode()))

    def set_geometry(self, mask: np.ndarray | None = None) -> None:
        """the base level's mask, or None for the record's analytic geometry"""
        if mask is None:
            _check(self._lib.lbm_set_geometry(self._h, None))
        else:
            self.set_mask(mask, 0)


SGS = {"none": 0, "smagorinsky": 1, "mlp": 2}


class Ensemble:
    """Periodic D3Q19 boxes of uneven sizes advanced together (one persistent
    launch per step, replayed from a CUDA graph); the data source and test bed
    of the learned subgrid closure."""

    def __init__(self, sizes, tau0, sgs: str = "none", cs: float = 0.01):
        self._lib = library()
        self.sizes = [int(n) for n in sizes]
        t = np.asarray(tau0 if np.ndim(tau0) else [tau0] * len(self.sizes), np.float32)
        self.tau0 = t
        sz = np.asarray(self.sizes, np.int32)
        h = _P()
        _check(self._lib.lbm_ensemble_create(len(sz), _ptr(sz), _ptr(t), SGS[sgs], _F(cs), ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lbm_ensemble_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init_turbulence(self, seed: int, u_rms: float = 0.04, kmax_div: int = 8, per_shell: int = 24) -> None:
        _check(self._lib.lbm_ensemble_init_turbulence(self._h, seed, _F(u_rms), kmax_div, per_shell))

    def modes(self, member: int):
        n = _I()
        _check(self._lib.lbm_ensemble_modes(self._h, member, None, None, None, 0, ctypes.byref(n)))
        k = np.zeros((n.value, 3), np.int32)
        ph = np.zeros(n.value)
        a = np.zeros((n.value, 3))
        _check(self._lib.lbm_ensemble_modes(self._h, member, _ptr(k), _ptr(ph), _ptr(a), n.value, ctypes.byref(n)))
        return k, ph, a

    def init_filtered(self, fine: "Ensemble") -> None:
        _check(self._lib.lbm_ensemble_init_filtered(self._h, fine._h))

    def set_mlp(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        _check(self._lib.lbm_ensemble_set_mlp(self._h, _ptr(p)))

    def autotune(self):
        ty, g, ms = _I(), _I(), _F()
        _check(self._lib.lbm_ensemble_autotune(self._h, ctypes.byref(ty), ctypes.byref(g), ctypes.byref(ms)))
        return ty.value, g.value, ms.value

    def step(self, n: int = 1) -> None:
        _check(self._lib.lbm_ensemble_step(self._h, n))

    def step_timed(self, n: int) -> float:
        ms = _F()
        _check(self._lib.lbm_ensemble_step_timed(self._h, n, ctypes.byref(ms)))
        return float(ms.value)

    def info(self) -> dict:
        ty, g, c, st = _I(), _I(), ctypes.c_longlong(), ctypes.c_longlong()
        _check(self._lib.lbm_ensemble_info(self._h, ctypes.byref(ty), ctypes.byref(g), ctypes.byref(c),
                                           ctypes.byref(st)))
        return dict(ty=ty.value, grid=g.value, cells=c.value, steps=st.value)

    def energy(self) -> np.ndarray:
        e = np.zeros(len(self.sizes))
        _check(self._lib.lbm_ensemble_energy(self._h, _ptr(e)))
        return e

    def velocity(self, member: int) -> np.ndarray:
        n = self.sizes[member]
        u = np.zeros((3, n, n, n), np.float32)
        _check(self._lib.lbm_ensemble_velocity(self._h, member, _ptr(u)))
        return u

    def populations(self, member: int) -> np.ndarray:
        n = self.sizes[member]
        f = np.zeros((19, n, n, n), np.float32)
        _check(self._lib.lbm_ensemble_populations(self._h, member, _ptr(f)))
        return f

    def set_populations(self, member: int, f: np.ndarray) -> None:
        g = np.ascontiguousarray(f, np.float32)
        _check(self._lib.lbm_ensemble_set_populations(self._h, member, _ptr(g)))

    def samples_into(self, X_ptr: int, T_ptr: int, cap: int, n: int = 0, tau0_coarse: float = 0.0) -> int:
        """append the filtered training samples of every member at device
        pointers X (float [cap][16]) and T (float [cap]); returns the new count"""
        c = ctypes.c_longlong(n)
        _check(self._lib.lbm_ensemble_samples(self._h, _F(tau0_coarse), _P(X_ptr), _P(T_ptr), cap, ctypes.byref(c)))
        return int(c.value)


def force_stats(fxyz, t_start: int, t_end: int | None = None):
    """ForceCalcs: mean and RMS per component of a force history (n, 3) over
    lines t_start .. t_end - 1, in the program's FP32 running arithmetic"""
    f = np.ascontiguousarray(fxyz, np.float32).reshape(-1, 3)
    n = f.shape[0]
    mean = np.zeros(3, np.float32)
    rms = np.zeros(3, np.float32)
    _check(library().lbm_force_stats(_ptr(f), n, t_start, n if t_end is None else t_end, _ptr(mean), _ptr(rms)))
    return mean, rms


def force_coefficients(fxyz, t_start: int, u: float, d: float, lz: float, rho: float = 1.0) -> dict:
    """C_D, RMS C_L and the Strouhal number of raw drag/lift histories (n, 3)"""
    f = np.ascontiguousarray(fxyz, np.float64).reshape(-1, 3)
    cd, cl, st = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _check(library().lbm_force_coefficients(_ptr(f), f.shape[0], t_start, u, d, lz, rho, ctypes.byref(cd),
                                            ctypes.byref(cl), ctypes.byref(st)))
    return dict(cd=cd.value, cl_rms=cl.value, st=st.value)


def wall_profile(v_mean, u_fluc, v_fluc, w_fluc, u_tau: float, nu: float) -> np.ndarray:
    """VelProf: rows (y+, v+, urms+, vrms+, wrms+) of a wall-normal line"""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (v_mean, u_fluc, v_fluc, w_fluc)]
    n = arrs[0].size
    out = np.zeros((5, n), np.float32)
    _check(library().lbm_wall_profile(*[_ptr(a) for a in arrs], n, _F(u_tau), _F(nu),
                                      *[_ptr(out[k]) for k in range(5)]))
    return out


def centerline_profiles(stats4: np.ndarray, umax: float) -> dict:
    """velplus: centre-line mean / RMS profiles of the plane z = nz / 2 of
    statistics float[4][nz][ny][nx], in units of umax"""
    s = np.ascontiguousarray(stats4, np.float32)
    _, nz, ny, nx = s.shape
    out = dict(uave=np.zeros(ny, np.float32), urms=np.zeros(ny, np.float32), vave=np.zeros(nx, np.float32),
               vrms=np.zeros(nx, np.float32))
    _check(library().lbm_centerline_profiles(_ptr(s), nx, ny, nz, umax, _ptr(out["uave"]),
                                             _ptr(out["urms"]), _ptr(out["vave"]), _ptr(out["vrms"])))
    return out


def stats_profiles(stats4: np.ndarray, x: int) -> np.ndarray:
    """profiles along y at x of statistics float[4][nz][ny][nx], z-averaged"""
    s = np.ascontiguousarray(stats4, np.float32)
    _, nz, ny, nx = s.shape
    out = np.zeros((4, ny), np.float32)
    _check(library().lbm_stats_profiles(_ptr(s), nx, ny, nz, x, _ptr(out)))
    return out
