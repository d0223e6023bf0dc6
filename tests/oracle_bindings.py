"""ctypes bindings of the CPU oracle (oracle/liblbm_oracle.so) and of the
staged reference harness (oracle/_ref/*.so).  Test infrastructure only: used
by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg, always as
the checker, never as the measured or shipped path.
"""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import ref_recipe  # noqa: E402

_P = ctypes.c_void_p
_F = ctypes.c_float
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1, 0, 1, 0, -1, 0, 0, 1, 0, -1, 0])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1, 0, 0, 1, 0, -1, 0, 0, 1, 0, -1])
CZ = np.array([0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1])
W = np.array([1 / 3] + [1 / 18] * 4 + [1 / 36] * 4 + [1 / 18] + [1 / 36] * 4 + [1 / 18] + [1 / 36] * 4)
# reference ImageFcn codes of the node types
REF_CODE = {0: 0, 1: 1, 2: 10, 3: 400, 4: 300, 5: 200, 6: 100}


def ptr(a: np.ndarray):
    return a.ctypes.data_as(_P)


class Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("model", ctypes.c_int),
                ("les", ctypes.c_int), ("omega", _F), ("cs", _F), ("dpdy", _F), ("u_in", _F), ("rho_out", _F),
                ("lid_u", _F * 3), ("lid_face", ctypes.c_int), ("force_on", ctypes.c_int),
                ("stats_on", ctypes.c_int), ("t", ctypes.c_int), ("start_av", ctypes.c_int),
                ("start_fluc", ctypes.c_int), ("stats_weight", _F), ("exp_x0", ctypes.c_int),
                ("exp_y0", ctypes.c_int), ("exp_nx", ctypes.c_int), ("exp_ny", ctypes.c_int),
                ("noise_amp", _F), ("noise_seed", ctypes.c_uint32), ("pull_clamp", ctypes.c_int),
                ("lid_quirk", ctypes.c_int), ("halfway", ctypes.c_int), ("mlp", ctypes.c_void_p),
                ("dyn_y1", ctypes.c_int), ("mlp_every", ctypes.c_int), ("mlp_nu", ctypes.c_void_p)]


class Refine(ctypes.Structure):
    _fields_ = [("cnx", ctypes.c_int), ("cny", ctypes.c_int), ("cnz", ctypes.c_int), ("fnx", ctypes.c_int),
                ("fny", ctypes.c_int), ("fnz", ctypes.c_int), ("lrx0", _F), ("lry0", _F), ("lrz0", _F),
                ("lrfactor", _F), ("lrlevel", ctypes.c_int), ("order", ctypes.c_int), ("cs", _F),
                ("omega_c", _F), ("omega_f", _F), ("quirk_fc_top_zflip", ctypes.c_int), ("zbounded", ctypes.c_int),
                ("cz0", ctypes.c_int)]


_oracle = None


def oracle() -> ctypes.CDLL:
    global _oracle
    if _oracle is None:
        _oracle = ctypes.CDLL(str(ref_recipe.build_oracle()))
        _oracle.orc_noise_uniform.restype = _F
        _oracle.orc_noise_hash.restype = ctypes.c_uint32
        _oracle.orc_mass.restype = ctypes.c_double
    return _oracle


def ref_lib(name: str) -> ctypes.CDLL | None:
    """The staged reference harness for a configuration, or None if absent."""
    p = ref_recipe.REF_DIR / name
    if not p.exists():
        if ref_recipe.staged():
            ref_recipe.build_ref()
        if not p.exists():
            return None
    return ctypes.CDLL(str(p))


def moments(f: np.ndarray):
    """rho, (jx, jy, jz) of populations [19, ...] in FP64"""
    g = f.astype(np.float64)
    return g.sum(0), np.stack([np.tensordot(c, g, 1) for c in (CX, CY, CZ)])


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


class OracleRun:
    """Oracle time loop for one configuration: the restated LR7 step sequence
    (coarse step, LRLEVEL fine sub-steps, InterpCF, InterpFC)."""

    def __init__(self, nx, ny, nz, mask, omega, *, model=0, les=0, cs=0.02, dpdy=0.0, u_in=0.05, init_kind=0,
                 init_u=0.05, lid_u=(0, 0, 0), lid_face=5, startf=0, refine=None, noise_amp=0.0, seed=12345,
                 stats=None, f0=None, pull_clamp=0, lid_quirk=0, halfway=0, mlp=None, cf_time=False, mlp_every=1):
        o = oracle()
        self.p = Params(nx=nx, ny=ny, nz=nz, model=model, les=les, omega=omega, cs=cs, dpdy=dpdy, u_in=u_in,
                        rho_out=1.0, lid_face=lid_face, stats_weight=1.0, noise_amp=noise_amp, noise_seed=seed,
                        pull_clamp=pull_clamp, lid_quirk=lid_quirk, halfway=halfway)
        if mlp is not None:
            self._mlp = np.ascontiguousarray(mlp, np.float32)
            self.p.mlp = self._mlp.ctypes.data
            if mlp_every > 1:
                self._nu = np.zeros(nx * ny * nz)
                self.p.mlp_every, self.p.mlp_nu = mlp_every, self._nu.ctypes.data
        self.p.lid_u[:] = list(lid_u)
        if stats:
            self.p.stats_on, self.p.start_av, self.p.start_fluc = 1, stats[0], stats[1]
            self.st = np.zeros((4, nz, ny, nx), np.float32)
        else:
            self.st = None
        self.mask = np.ascontiguousarray(mask, np.uint8)
        self.fa = np.zeros((19, nz, ny, nx), np.float32)
        o.orc_init(ctypes.byref(self.p), ptr(self.mask), ptr(self.fa), init_kind, _F(init_u))
        if f0 is not None:
            self.fa[:] = f0
        self.fb = self.fa.copy()
        self.startf = startf
        self.t = 0
        self.forces = []
        self.refine = refine
        if refine is not None:
            r, fmask, omega_f, f0f = refine["r"], refine["mask"], refine["omega_f"], refine.get("f0")
            self.r = r
            self.fmask = np.ascontiguousarray(fmask, np.uint8)
            self.pf = Params(nx=r.fnx, ny=r.fny, nz=r.fnz, model=model, les=les, omega=omega_f, cs=cs, dpdy=dpdy,
                             u_in=u_in, rho_out=1.0, stats_weight=r.lrfactor)
            self.ffa = np.zeros((19, r.fnz, r.fny, r.fnx), np.float32)
            o.orc_init(ctypes.byref(self.pf), ptr(self.fmask), ptr(self.ffa), init_kind, _F(init_u))
            if f0f is not None:
                self.ffa[:] = f0f
            self.ffb = self.ffa.copy()
            enx, eny = int(r.fnx * r.lrfactor) + 1, int(r.fny * r.lrfactor) + 1
            self.p.exp_x0, self.p.exp_y0, self.p.exp_nx, self.p.exp_ny = int(r.lrx0), int(r.lry0), enx, eny
            self.mom = np.zeros((9, nz, eny, enx), np.float32)
            # linear temporal interpolation of the band (CF TIME: linear)
            self.cf_time, self.have_mom = cf_time, False
            self.mom_prev = np.zeros_like(self.mom)

    def step(self, n=1):
        o = oracle()
        for _ in range(n):
            t = self.t
            self.p.t = t
            self.p.force_on = 1 if (self.refine is None and t > self.startf) else 0
            f3 = np.zeros(3)
            st = [ptr(self.st[i]) for i in range(4)] if self.st is not None else [None] * 4
            blend = False
            if self.refine is not None and self.cf_time:
                self.mom, self.mom_prev = self.mom_prev, self.mom
                blend, self.have_mom = self.have_mom, True
            o.orc_step(ctypes.byref(self.p), ptr(self.mask), ptr(self.fa), ptr(self.fb), ptr(f3), *st,
                       ptr(self.mom) if self.refine is not None else None)
            self.fa, self.fb = self.fb, self.fa
            if self.refine is not None:
                L = self.r.lrlevel
                for i in range(L):
                    if blend and i > 0:
                        th = np.float32(i / L)
                        mb = np.ascontiguousarray((np.float32(1) - th) * self.mom_prev + th * self.mom, np.float32)
                        o.orc_interp_cf(ctypes.byref(self.r), ptr(mb), ptr(self.ffa), ptr(self.fmask))
                    self.pf.t = t
                    self.pf.force_on = 1 if (t > self.startf and i == 0) else 0
                    o.orc_step(ctypes.byref(self.pf), ptr(self.fmask), ptr(self.ffa), ptr(self.ffb), ptr(f3),
                               None, None, None, None, None)
                    self.ffa, self.ffb = self.ffb, self.ffa
                o.orc_interp_cf(ctypes.byref(self.r), ptr(self.mom), ptr(self.ffa), ptr(self.fmask))
                o.orc_interp_fc(ctypes.byref(self.r), ptr(self.ffa), ptr(self.fa), ptr(self.mask))
            if t >= self.startf:
                self.forces.append(f3.copy())
            self.t += 1
