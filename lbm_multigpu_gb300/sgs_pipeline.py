"""Training pipeline of the learned subgrid closure, end to end on one GPU.

1. Data: a seeded ensemble of decaying-turbulence periodic boxes of uneven
   sizes (random-phase solenoidal field, E(k) ~ k^-5/3, u_rms 0.04) run
   with molecular viscosity only at 2x resolution, all members advanced by
   one persistent launch per step from a CUDA graph (tile shape and grid
   from the autotuner).  At a few times every member is box-filtered 2x2x2
   onto the coarse grid; each coarse cell gives a sample: the features of
   its resolved stress and the least-squares eddy viscosity of the filtered
   subgrid stress (lbm_ensemble_samples).
2. Training: the fused forward/backward and Adam kernels (lbm_mlp_train),
   on the coefficient o = nu / (x12 / tau0) of each sample: the collision
   takes nu_t = o x12 / tau0 = o 100 |S|, a local Smagorinsky coefficient
   (coefficient_targets).
3. Evaluation (a posteriori): held-out boxes run at coarse resolution from
   the filtered initial field with no model, with Smagorinsky (Cs = 0.1)
   and with the learned closure, against the filtered 2x-resolution run:
   kinetic-energy history and the energy spectrum.

Acoustic scaling between the grids: same lattice velocity, dt_c = 2 dt_f,
nu_f (lattice) = 2 nu_c (lattice), so tau_f - 1/2 = 2 (tau_c - 1/2) and one
coarse step is two fine steps.

4. The same three closures in the square-cylinder channel against its 2x
   run (channel_profiles): mean-velocity and fluctuation profiles behind
   the cylinder, held out on the benchmarked 512 x 128 x 128 channel
   (tau0 = 0.52, side 16) with a 1024 x 256 x 256 reference.  The
   training adds samples of 2x channels at tau0 = 0.505 and 0.52, with the
   regularised least-squares targets of samples_from_velocity.

Run:  python -m lbm_multigpu_gb300.sgs_pipeline --out weights.bin
      python -m lbm_multigpu_gb300.sgs_pipeline channel --weights weights.bin
"""
from __future__ import annotations

import argparse
import ctypes
import json
import time

import numpy as np

from . import Ensemble, _check, _ptr, library

TAU_C = 0.505              # coarse molecular relaxation time (nu_c = 1/600); the 2x run at
                           # tau_f = 0.51 stays stable for the 5-sigma velocity peaks of u_rms 0.04
TAU_F = 0.5 + 2 * (TAU_C - 0.5)
CS = 0.01                  # Smagorinsky CS = Cs^2, Cs = 0.1


def ensemble_sizes(seed: int, count: int = 16, lo: int = 64, hi: int = 160, step: int = 16) -> list[int]:
    """uneven fine box sides drawn by seed from lo..hi (multiples of step)"""
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.choice(np.arange(lo, hi + 1, step), size=count)]


def generate(sizes: list[int], seed: int, snapshots=(100, 200, 300, 400, 500, 600), u_rms: float = 0.04):
    """samples (torch CUDA tensors X [n,16], T [n]) and a timing record"""
    import torch

    cap = len(snapshots) * sum((n // 2) ** 3 for n in sizes)
    X = torch.empty((cap, 16), dtype=torch.float32, device="cuda")
    T = torch.empty(cap, dtype=torch.float32, device="cuda")
    info = {}
    with Ensemble(sizes, TAU_F, sgs="none") as fine:
        fine.init_turbulence(seed, u_rms=u_rms, kmax_div=8, per_shell=24)
        ty, grid, ms_tuned = fine.autotune()
        cells = fine.info()["cells"]
        n, t_prev, ms_total, steps_total = 0, 0, 0.0, 0
        for tc in snapshots:                       # coarse-step times
            k = 2 * (tc - t_prev)
            ms_total += fine.step_timed(k)
            steps_total += k
            t_prev = tc
            n = fine.samples_into(X.data_ptr(), T.data_ptr(), cap, n, TAU_C)
        info = dict(members=len(sizes), sizes=sizes, cells=cells, ty=ty, grid=grid, fine_steps=steps_total,
                    ms_per_step=ms_total / steps_total, mlups=cells * steps_total / (ms_total * 1e3), samples=n)
    return X[:n], T[:n], info


def coefficient_targets(X, T, o_max: float = 5e-3):
    """the network's targets from eddy-viscosity targets T of samples X: the
    coefficient o = T / (x12 / tau0) (the collision uses nu_t = o x12 / tau0,
    o 100 |S|), 0 where x12 is 0, at most o_max (Cs^2 = 0.5; the
    least-squares fit divides by the strain, so cells of weak strain can give
    outliers).  Torch tensors or numpy arrays."""
    tau0 = X[:, 14] / 100 + 0.5
    g = X[:, 12] / tau0
    if isinstance(T, np.ndarray):
        with np.errstate(divide="ignore", invalid="ignore"):
            return np.where(g > 0, np.minimum(T / g, o_max), 0.0).astype(T.dtype)
    import torch

    return torch.where(g > 0, torch.clamp(T / torch.clamp(g, min=1e-30), max=o_max), torch.zeros_like(T))


def train(X, T, steps: int = 4000, batch: int = 16384, lr: float = 2e-3, seed: int = 1, scale: float = 1.0):
    """the MLP trained on targets scale * T"""
    lib = library()
    if scale != 1.0:
        T = T * scale
    P = np.zeros(lib.lbm_mlp_param_count(), np.float32)
    _check(lib.lbm_mlp_init_params(seed, _ptr(P)))
    # start the output near the mean target: softplus(b3) = mean(T) / 1e-4
    m = max(float(T.mean().item()) / 1e-4, 1e-3)
    P[-1] = float(np.log(np.expm1(m)))
    hist = np.zeros(steps, np.float32)
    t0 = time.perf_counter()
    _check(lib.lbm_mlp_train(ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(T.data_ptr()), int(X.shape[0]), batch,
                             steps, ctypes.c_float(lr), seed, _ptr(P), _ptr(hist), None))
    return P, hist, time.perf_counter() - t0


def _filtered_energy_spectrum(u: np.ndarray):
    """energy of the 2x2x2-filtered velocity and its shell spectrum"""
    n = u.shape[1]
    ub = u.reshape(3, n // 2, 2, n // 2, 2, n // 2, 2).mean(axis=(2, 4, 6))
    return _energy_spectrum(ub)


def _energy_spectrum(u: np.ndarray):
    n = u.shape[1]
    uk = np.fft.fftn(u, axes=(1, 2, 3)) / n ** 3
    e = 0.5 * (np.abs(uk) ** 2).sum(0)
    k = np.fft.fftfreq(n, 1.0 / n)
    kk = np.sqrt(k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2)
    shells = np.rint(kk).astype(int)
    spec = np.bincount(shells.ravel(), e.ravel(), minlength=n // 2 + 1)[: n // 2 + 1]
    return float(0.5 * (u ** 2).sum(0).mean()), spec


def evaluate(params: np.ndarray, sizes: list[int], seed: int, coarse_steps: int = 600, every: int = 50,
             models=("none", "smagorinsky", "mlp")):
    """a-posteriori comparison: relative errors of the energy history and of
    the upper half of the final spectrum against the filtered 2x run, for no
    model, Smagorinsky and the learned closure"""
    csizes = [n // 2 for n in sizes]
    fine = Ensemble(sizes, TAU_F, sgs="none")
    fine.init_turbulence(seed, kmax_div=8, per_shell=24)
    runs = {name: Ensemble(csizes, TAU_C, sgs=name, cs=CS) for name in models}
    if "mlp" in runs:
        runs["mlp"].set_mlp(params)
    for e in runs.values():
        e.init_filtered(fine)
    hist = {k: [] for k in ("truth", *runs)}
    for t in range(every, coarse_steps + 1, every):
        fine.step(2 * every)
        for e in runs.values():
            e.step(every)
        hist["truth"].append([_filtered_energy_spectrum(fine.velocity(m))[0] for m in range(len(sizes))])
        for k, e in runs.items():
            hist[k].append(list(e.energy()))
    spec_truth = [_filtered_energy_spectrum(fine.velocity(m))[1] for m in range(len(sizes))]
    out = {}
    truth = np.array(hist["truth"])
    if not np.isfinite(truth).all():
        raise FloatingPointError(f"the 2x reference run of seed {seed} went unstable")
    for k, e in runs.items():
        h = np.array(hist[k])
        err_e = float(np.linalg.norm(h - truth) / np.linalg.norm(truth))
        errs = []
        for m, n in enumerate(csizes):
            s = _energy_spectrum(e.velocity(m))[1]
            lo, hi = n // 8, n // 2
            st = spec_truth[m][lo:hi]
            errs.append(float(np.linalg.norm(np.log(s[lo:hi] + 1e-30) - np.log(st + 1e-30)) / np.sqrt(hi - lo)))
        out[k] = dict(energy_rel_l2=err_e, spectrum_log_rms=float(np.mean(errs)))
    out["truth_energy_final"] = [float(v) for v in truth[-1]]
    fine.close()
    for e in runs.values():
        e.close()
    return out


def features_np(p: np.ndarray, tau0: float) -> np.ndarray:
    """the closure's 16 inputs (as the collide kernel forms them, sgs_mlp.cuh)
    of p_ij = [xx, yy, zz, xy, xz, yz] (shape (6, n)), in float64"""
    P_REF = 0.01
    xx, yy, zz, xy, xz, yz = p
    pp = xx * xx + yy * yy + zz * zz + 2 * (xy * xy + xz * xz + yz * yz)
    tr3 = (xx ** 3 + yy ** 3 + zz ** 3 + 3 * xx * (xy * xy + xz * xz) + 3 * yy * (xy * xy + yz * yz) +
           3 * zz * (xz * xz + yz * yz) + 6 * xy * xz * yz)
    x = np.empty((16, p.shape[1]))
    x[0:12] = 0.0                 # reserved: invariants of p only
    x[12] = np.sqrt(2 * pp) / P_REF
    with np.errstate(divide="ignore", invalid="ignore"):
        x[13] = np.where(pp > 1e-30, tr3 / (pp * np.sqrt(np.maximum(pp, 1e-300))), 0.0)
    x[14] = (tau0 - 0.5) * 100
    x[15] = 1.0
    return x.T


def samples_from_velocity(u: np.ndarray, fluid: np.ndarray, tau0: float, margin: int = 2, reg: float = 0.0):
    """training samples of a 2x-resolution field that is periodic in z only:
    u float[3][fz][fy][fx] and fluid bool[fz][fy][fx] (nodes that are plain
    fluid).  As the ensemble's samples (2x2x2 box filter, central-difference
    strain of the filtered velocity, the deviatoric subgrid stress, 3x3x3
    averages of tau^d:S and S:S, features of p = (tau0 + 3 nu) S), on the
    coarse cells whose filter boxes, and those of their neighbours up to
    `margin` cells in x and y, hold fluid only.  The eddy viscosity is the
    regularised least-squares fit nu = max(0, -<tau^d:S>) / (2 (<S:S> + eps))
    with eps = reg * (mean <S:S> over those cells): with reg > 0 it goes to
    zero where the strain is weak against the flow's (a channel's free
    stream, where <tau^d:S> and <S:S> are both at the level of the inlet
    noise and their ratio is noise); reg = 0 is the plain fit of the
    ensemble's samples.  Returns X float32[n][16], T float32[n]."""
    _, fz, fy, fx = u.shape
    cz, cy, cx = fz // 2, fy // 2, fx // 2

    def box(a):
        return a.reshape(a.shape[:-3] + (cz, 2, cy, 2, cx, 2)).mean(axis=(-5, -3, -1))

    ub = box(u.astype(np.float64))
    uu = box(np.stack([u[0] * u[0], u[1] * u[1], u[2] * u[2], u[0] * u[1], u[0] * u[2], u[1] * u[2]]).astype(np.float64))
    ok = box(fluid.astype(np.float64)) == 1.0

    def d(a, axis):
        return 0.5 * (np.roll(a, -1, axis) - np.roll(a, 1, axis))

    g = np.stack([np.stack([d(ub[k], 2), d(ub[k], 1), d(ub[k], 0)]) for k in range(3)])  # g[k][axis x,y,z]
    S = np.stack([g[0, 0], g[1, 1], g[2, 2], 0.5 * (g[0, 1] + g[1, 0]), 0.5 * (g[0, 2] + g[2, 0]),
                  0.5 * (g[1, 2] + g[2, 1])])
    tau = uu - np.stack([ub[0] * ub[0], ub[1] * ub[1], ub[2] * ub[2], ub[0] * ub[1], ub[0] * ub[2], ub[1] * ub[2]])
    tau[:3] -= tau[:3].sum(0) / 3
    w = np.array([1, 1, 1, 2, 2, 2], np.float64)[:, None, None, None]
    ts, ss = (w * tau * S).sum(0), (w * S * S).sum(0)

    def avg3(a):
        out = np.zeros_like(a)
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    out += np.roll(a, (dz, dy, dx), axis=(0, 1, 2))
        return out

    ts, ss = avg3(ts), avg3(ss)
    valid = ok.copy()
    for dy in range(-margin, margin + 1):
        for dx in range(-margin, margin + 1):
            valid &= np.roll(ok, (dy, dx), axis=(1, 2))
    if margin > 0:
        valid[:, :margin, :] = valid[:, -margin:, :] = False
        valid[:, :, :margin] = valid[:, :, -margin:] = False
    eps = reg * float(ss[valid].mean()) if valid.any() else 0.0
    with np.errstate(divide="ignore", invalid="ignore"):
        nu = np.where(ss + eps > 1e-30, np.maximum(-ts, 0.0) / (2 * (ss + eps)), 0.0)
    nu = nu[valid]
    p = (tau0 + 3 * nu) * S[:, valid]
    return features_np(p, tau0).astype(np.float32), nu.astype(np.float32)


def _channel_record(nx: int, ny: int, nz: int, centre: tuple[float, float], half: float, tau: float, sgs: str,
                    tmax: int, seed: int, stats: tuple[int, int] | None = None, sgs_every: int = 1) -> str:
    """the square-cylinder channel (MRT, half-way walls, inlet 0.05 with 1 %
    seeded noise); stats = (start of the mean, start of the variance);
    sgs_every: the closure's refresh interval"""
    from . import make_inputs

    kw = dict(sgs="mlp", sgs_every=sgs_every) if sgs == "mlp" else {}
    if stats:
        kw.update(velav=1, start_velav=stats[0], start_velfluc=stats[1])
    return make_inputs(nx, ny, nz, obst1=(centre[0], centre[1], 0.0), r1=half, umax=0.05, tmax=tmax,
                       les=0 if sgs == "none" else 1, cs=CS, model="MRT", geometry="channel_square", tau=tau,
                       inlet_noise=0.01, seed=seed, bounceback="halfway", **kw)


def _channel_geometry(coarse, side: int, centre_x: int | None = None):
    """coarse centre (a node boundary on both axes: x = centre_x + 1/2, by
    default nx / 6) and half side"""
    nx, ny, _ = coarse
    return ((nx // 6 if centre_x is None else centre_x) + 0.5, ny // 2 - 0.5), side / 2


def fine_tau(tau_c: float) -> float:
    """relaxation time of the 2x grid under acoustic scaling"""
    return 0.5 + 2 * (tau_c - 0.5)


def _channel_run(nx: int, ny: int, nz: int, centre: tuple[float, float], half: float, tau: float, sgs: str,
                 params, spinup: int, mean_steps: int, fluc_steps: int, seed: int, chunk: int = 2000,
                 sgs_every: int = 1):
    """one channel run with running statistics: the mean over
    [spinup, spinup + mean_steps), the variance about it over the next
    fluc_steps.  Returns the statistics, or None if the run blew up."""
    from . import Solver

    t_end = spinup + mean_steps + fluc_steps
    text = _channel_record(nx, ny, nz, centre, half, tau, sgs, t_end, seed, (spinup, spinup + mean_steps),
                           sgs_every)
    with Solver(text) as s:
        if sgs == "mlp":
            s.set_sgs_mlp(params)
        t = 0
        while t < t_end:
            k = min(chunk, t_end - t)
            s.step(k)
            t += k
        st = s.stats()
    return st if np.isfinite(st).all() else None


def generate_channel(coarse=(160, 64, 32), side: int = 8, seed: int = 777, spinup: int = 6000, snapshots: int = 12,
                     every: int = 500, tau_c: float = TAU_C, centre_x: int | None = None, reg: float = 0.0):
    """training samples from the square-cylinder channel at 2x resolution
    (fine_tau(tau_c), no model), taken every `every` coarse steps after
    `spinup`; the features carry tau_c; reg: samples_from_velocity"""
    import torch

    from . import Solver

    nx, ny, nz = coarse
    (cx, cy), half = _channel_geometry(coarse, side, centre_x)
    t_end = 2 * (spinup + snapshots * every)
    text = _channel_record(2 * nx, 2 * ny, 2 * nz, (2 * cx + 0.5, 2 * cy + 0.5), 2 * half, fine_tau(tau_c), "none",
                           t_end, seed)
    Xs, Ts = [], []
    t0 = time.perf_counter()
    with Solver(text) as s:
        fluid = s.mask() == 0
        s.step(2 * spinup)
        for _ in range(snapshots):
            s.step(2 * every)
            rho, jx, jy, jz = s.fields()
            if not np.isfinite(rho).all():
                raise FloatingPointError("the 2x channel run for training went unstable")
            X, T = samples_from_velocity(np.stack([jx, jy, jz]) / rho, fluid, tau_c, reg=reg)
            Xs.append(X)
            Ts.append(T)
    X, T = np.concatenate(Xs), np.concatenate(Ts)
    info = dict(coarse=list(coarse), side=side, seed=seed, spinup=spinup, snapshots=snapshots, every=every,
                tau_c=tau_c, centre_x=centre_x, reg=reg, samples=int(len(T)), target_mean=float(T.mean()),
                seconds=time.perf_counter() - t0)
    return torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda(), info


def channel_truth(coarse=(192, 64, 32), side: int = 8, spinup: int = 4000, mean_steps: int = 4000,
                  fluc_steps: int = 4000, stations=(1, 2, 4, 8), seed: int = 12345, tau_c: float = TAU_C,
                  centre_x: int | None = None) -> dict:
    """the reference of the channel comparison: the square cylinder of side
    `side` in a channel on the 2x grid (tau_f = fine_tau(tau_c), molecular
    viscosity only, twice the steps), its statistics box-filtered 2 x 2 in x
    and y (z is averaged) onto the coarse stations `stations` cylinder sides
    behind the rear face.  Profiles along y: mean u, mean v, variance of u,
    variance of v (truth: float[stations][4][ny])."""
    from . import stats_profiles

    nx, ny, nz = coarse
    (cx, cy), half = _channel_geometry(coarse, side, centre_x)
    fine = _channel_run(2 * nx, 2 * ny, 2 * nz, (2 * cx + 0.5, 2 * cy + 0.5), 2 * half, fine_tau(tau_c), "none",
                        None, 2 * spinup, 2 * mean_steps, 2 * fluc_steps, seed)
    if fine is None:
        raise FloatingPointError("the 2x reference channel run went unstable")
    rear = int(np.floor(cx + half))                     # last coarse node inside the cylinder
    xs = [rear + k * side for k in stations if rear + k * side < nx - 1]

    def fine_profile(x: int) -> np.ndarray:
        p = 0.5 * (stats_profiles(fine, 2 * x) + stats_profiles(fine, 2 * x + 1))   # (4, 2 ny)
        return p.reshape(4, ny, 2).mean(axis=2)

    return dict(truth=np.stack([fine_profile(x) for x in xs]), stations=xs, coarse=tuple(coarse), side=side,
                steps=(spinup, mean_steps, fluc_steps), seed=seed, tau_c=tau_c, centre_x=centre_x)


def zero_closure(params) -> np.ndarray:
    """the closure's weights with the output bias at -30: the coefficient
    1e-4 softplus(-30), and so nu_t, zero to FP32 precision"""
    z = np.array(params if params is not None and len(params) else np.zeros(library().lbm_mlp_param_count()),
                 np.float32)
    z[-1] = -30.0
    return z


def channel_errors(params, ref: dict, models=("none", "smagorinsky", "mlp"), sgs_every: int = 1):
    """the coarse runs of `models` (tau0 = ref["tau_c"]) against `ref`
    (channel_truth): relative L2 of the mean-u, u-rms and v-rms profiles
    (walls excluded), "unstable" for a run that blew up; and the profiles.
    Model "spread" is the closure kernel with zero eddy viscosity
    (zero_closure): its errors are measured against the "none" run (same
    physics, FP32 rounding apart), so they show how far the statistics of
    this run length move from a rounding-level perturbation alone.
    sgs_every: the closure's refresh interval (SGS every)."""
    from . import stats_profiles

    nx, ny, nz = ref["coarse"]
    (cx, cy), half = _channel_geometry(ref["coarse"], ref["side"], ref.get("centre_x"))
    tau_c = ref.get("tau_c", TAU_C)
    truth, inner = ref["truth"], slice(1, ny - 1)

    def rel(a: np.ndarray, b: np.ndarray) -> float:
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    rms_t = np.sqrt(np.maximum(truth[:, 2:4], 0.0))
    out, profiles = {}, {}
    for name in models:
        sgs, w = ("mlp", zero_closure(params)) if name == "spread" else (name, params)
        st = _channel_run(nx, ny, nz, (cx, cy), half, tau_c, sgs, w, *ref["steps"], ref["seed"],
                          sgs_every=sgs_every if name == "mlp" else 1)
        if st is None:
            out[name] = "unstable"
            continue
        prof = np.stack([stats_profiles(st, x) for x in ref["stations"]])
        profiles[name] = prof
        if name == "spread":
            continue
        rms = np.sqrt(np.maximum(prof[:, 2:4], 0.0))
        out[name] = dict(u_mean_rel_l2=rel(prof[:, 0, inner], truth[:, 0, inner]),
                         u_rms_rel_l2=rel(rms[:, 0, inner], rms_t[:, 0, inner]),
                         v_rms_rel_l2=rel(rms[:, 1, inner], rms_t[:, 1, inner]))
    if "spread" in profiles and "none" in profiles:
        a, b = profiles["spread"], profiles["none"]
        ra, rb = np.sqrt(np.maximum(a[:, 2:4], 0.0)), np.sqrt(np.maximum(b[:, 2:4], 0.0))
        # in units of the truth's norms, so that they compare with the errors above
        out["spread"] = dict(u_mean_rel_l2=float(np.linalg.norm(a[:, 0, inner] - b[:, 0, inner])
                                                 / np.linalg.norm(truth[:, 0, inner])),
                             u_rms_rel_l2=float(np.linalg.norm(ra[:, 0, inner] - rb[:, 0, inner])
                                                / np.linalg.norm(rms_t[:, 0, inner])),
                             v_rms_rel_l2=float(np.linalg.norm(ra[:, 1, inner] - rb[:, 1, inner])
                                                / np.linalg.norm(rms_t[:, 1, inner])))
    return out, profiles


def channel_profiles(params: np.ndarray, coarse=(192, 64, 32), side: int = 8, spinup: int = 4000,
                     mean_steps: int = 4000, fluc_steps: int = 4000, stations=(1, 2, 4, 8), seed: int = 12345,
                     models=("none", "smagorinsky", "mlp", "spread"), tau_c: float = TAU_C,
                     centre_x: int | None = None, sgs_every: int = 1):
    """a-posteriori comparison in the square-cylinder channel family: a
    square cylinder in a channel (coarse grid `coarse`, tau0 = tau_c, i.e.
    Re = 3 * 0.05 * side / (tau_c - 1/2)) run with no model, Smagorinsky and
    the learned closure, against the same channel at 2x resolution
    (channel_truth).  Returns the errors (channel_errors) with the setup, and
    the profiles (the reference as "truth").  The benchmarked channel is
    coarse=(512, 128, 128), side=16, tau_c=0.52, centre_x=128.

    The fine walls sit half a coarse cell outside the coarse ones (both
    grids put the half-way wall half a spacing off their first node); the
    fine variances include the fluctuations below the coarse filter width."""
    ref = channel_truth(coarse, side, spinup, mean_steps, fluc_steps, stations, seed, tau_c, centre_x)
    out = dict(stations=ref["stations"], coarse=list(coarse), side=side, centre_x=centre_x, tau_c=tau_c,
               tau_f=fine_tau(tau_c), re=3 * 0.05 * side / (tau_c - 0.5), steps=[spinup, mean_steps, fluc_steps],
               sgs_every=sgs_every)
    errs, profiles = channel_errors(params, ref, models, sgs_every)
    out.update(errs)
    profiles["truth"] = ref["truth"]
    return out, profiles


def calibrate(X, T, sizes: list[int], seed: int, alphas, steps: int, batch: int, lr: float, train_seed: int,
              channel_refs=()):
    """scale of the training targets chosen a posteriori on configurations
    of the training data (the least-squares eddy viscosity of the filtered
    stress is an a-priori estimate; the coarse solver has numerical
    dissipation of its own).  Score of a scale: the filtered-2x energy-history
    error on the training-seed boxes relative to Smagorinsky's, plus, for
    each of `channel_refs` (channel_truth of the training channels), the
    mean-u and u-rms profile errors relative to Smagorinsky's there.  Lowest
    score wins."""
    base = evaluate(np.zeros(0, np.float32), sizes, seed, coarse_steps=600, models=("smagorinsky",))
    iso_smag = base["smagorinsky"]["energy_rel_l2"]
    chan_smag = []
    for ref in channel_refs:
        cs_err, _ = channel_errors(None, ref, ("smagorinsky",))
        chan_smag.append(cs_err["smagorinsky"]["u_mean_rel_l2"] + cs_err["smagorinsky"]["u_rms_rel_l2"])
    res = []
    for a in alphas:
        P, hist, _ = train(X, T, steps, batch, lr, train_seed, scale=a)
        ev = evaluate(P, sizes, seed, coarse_steps=600, models=("mlp",))
        parts = dict(iso=ev["mlp"]["energy_rel_l2"] / iso_smag)
        for i, ref in enumerate(channel_refs):
            ce, _ = channel_errors(P, ref, ("mlp",))
            m = ce["mlp"]
            parts[f"channel{i}"] = ((m["u_mean_rel_l2"] + m["u_rms_rel_l2"]) / chan_smag[i] if isinstance(m, dict)
                                    else np.inf)
        score = float(sum(parts.values()))
        res.append((score if np.isfinite(score) else np.inf, a, P, hist, parts))
    res.sort(key=lambda r: r[0])
    table = [dict(alpha=float(a), score=float(sc), **{k: float(v) for k, v in pt.items()})
             for sc, a, _, _, pt in res]
    return res[0][1], res[0][2], res[0][3], table


# training channels: the square cylinder at Re 240 (side 8, tau0 0.505) and
# at the benchmarked channel's Re 120 (side 16, tau0 0.52) on a shallower grid
DEFAULT_TRAIN_CHANNELS = "160x64x32,8,0.505,-1;320x128x32,16,0.52,80"
# held out: Re 240 on another grid, and the benchmarked channel itself
DEFAULT_EVAL_CHANNELS = "192x64x32,8,0.505,-1,6000,30000,30000;512x128x128,16,0.52,128,6000,12000,12000"


def parse_channels(text: str) -> list[tuple]:
    """';'-separated channel specs NXxNYxNZ,side,tau0,centre_x[,spin-up,mean,
    fluctuation] (centre_x -1: nx / 6)"""
    out = []
    for spec in filter(None, (t.strip() for t in text.split(";"))):
        f = spec.split(",")
        coarse = tuple(int(v) for v in f[0].split("x"))
        cx = int(f[3]) if len(f) > 3 and int(f[3]) >= 0 else None
        out.append((coarse, int(f[1]), float(f[2]), cx, *(int(v) for v in f[4:7])))
    return out


def channel_main(argv) -> int:
    """python -m lbm_multigpu_gb300.sgs_pipeline channel --weights W [--report R]"""
    ap = argparse.ArgumentParser(description="learned closure vs Smagorinsky in the square-cylinder channel")
    ap.add_argument("--weights", required=True, help="float32 parameter file")
    ap.add_argument("--coarse", default="192x64x32")
    ap.add_argument("--side", type=int, default=8)
    ap.add_argument("--steps", default="4000,4000,4000", help="spin-up, mean, fluctuation coarse steps")
    ap.add_argument("--tau", type=float, default=TAU_C, help="coarse tau0")
    ap.add_argument("--centre-x", type=int, default=None, help="cylinder centre x (coarse node; default nx/6)")
    ap.add_argument("--sgs-every", type=int, default=1, help="the closure's refresh interval (SGS every)")
    ap.add_argument("--seed", type=int, default=12345)
    ap.add_argument("--report", default=None, help="JSON report path")
    ap.add_argument("--profiles", default=None, help=".npz of the profiles")
    a = ap.parse_args(argv)
    P = np.fromfile(a.weights, dtype="<f4")
    coarse = tuple(int(v) for v in a.coarse.split("x"))
    sp, ms, fs = (int(v) for v in a.steps.split(","))
    t0 = time.perf_counter()
    out, prof = channel_profiles(P, coarse, a.side, sp, ms, fs, seed=a.seed, tau_c=a.tau, centre_x=a.centre_x,
                                 sgs_every=a.sgs_every)
    out["seconds"] = time.perf_counter() - t0
    out["weights"] = a.weights
    print(json.dumps(out))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(out, f, indent=1)
    if a.profiles:
        np.savez_compressed(a.profiles, **prof)
    return 0


def main(argv=None) -> int:
    import sys

    argv = sys.argv[1:] if argv is None else argv
    if argv and argv[0] == "channel":
        return channel_main(argv[1:])
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", required=True, help="float32 parameter file (lbm_mlp_param_count values)")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--members", type=int, default=16)
    ap.add_argument("--train-steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--eval-sizes", default="64,96,128,160")
    ap.add_argument("--report", default=None, help="JSON report path")
    ap.add_argument("--alphas", default="0.2,0.3,0.4,0.5,0.6,0.7,0.85,1.0",
                    help="candidate target scales for the a-posteriori calibration")
    ap.add_argument("--channel-train", default=DEFAULT_TRAIN_CHANNELS,
                    help="training channels, ';'-separated NXxNYxNZ,side,tau0,centre_x ('' for isotropic boxes only)")
    ap.add_argument("--channel-seed", type=int, default=777)
    ap.add_argument("--channel-eval", default=DEFAULT_EVAL_CHANNELS,
                    help="held-out channels, ';'-separated NXxNYxNZ,side,tau0,centre_x,spin-up,mean,fluctuation")
    ap.add_argument("--channel-eval-seed", type=int, default=12345)
    ap.add_argument("--channel-steps", default="6000,20000,20000",
                    help="spin-up, mean, fluctuation coarse steps of the calibration channels")
    ap.add_argument("--channel-reg", type=float, default=0.25,
                    help="regularisation of the channel targets (samples_from_velocity reg)")
    a = ap.parse_args(argv)
    import torch

    sizes = ensemble_sizes(a.seed, a.members)
    X, T, gen = generate(sizes, a.seed)
    ch_steps = tuple(int(v) for v in a.channel_steps.split(","))
    chan_gen, chan_refs = [], []
    for i, spec in enumerate(parse_channels(a.channel_train)):
        coarse, side, tau_c, cx = spec[:4]
        Xc, Tc, info = generate_channel(coarse, side, seed=a.channel_seed + i, tau_c=tau_c, centre_x=cx,
                                        reg=a.channel_reg)
        X, T = torch.cat([X, Xc]), torch.cat([T, Tc])
        chan_gen.append(info)
        chan_refs.append(channel_truth(coarse, side, *ch_steps, seed=a.channel_seed + i, tau_c=tau_c, centre_x=cx))
    T = coefficient_targets(X, T)
    t0 = time.perf_counter()
    eval_sizes = [int(v) for v in a.eval_sizes.split(",")]
    # calibration: the evaluation sizes with the training seed's fields, and
    # the training channels
    alpha, P, hist, table = calibrate(X, T, eval_sizes, a.seed, [float(v) for v in a.alphas.split(",")],
                                      a.train_steps, a.batch, a.lr, a.seed, chan_refs)
    secs = time.perf_counter() - t0
    P.astype("<f4").tofile(a.out)
    # held out: a different seed for the initial fields, other channels
    ev = evaluate(P, eval_sizes, a.seed + 1)
    ch_eval = []
    for coarse, side, tau_c, cx, *steps in parse_channels(a.channel_eval):
        out, _ = channel_profiles(P, coarse, side, *(steps or ch_steps), seed=a.channel_eval_seed, tau_c=tau_c,
                                  centre_x=cx)
        ch_eval.append(out)
    rep = dict(generate=gen, generate_channel=chan_gen,
               train=dict(steps=a.train_steps, batch=a.batch, lr=a.lr, seconds_with_calibration=secs,
                          alpha=alpha, calibration=table, loss_first=float(hist[:10].mean()),
                          loss_last=float(hist[-50:].mean()), target_mean=float(T.mean().item()),
                          target_std=float(T.std().item()), samples=int(T.shape[0])),
               evaluate=ev, evaluate_channel=ch_eval, weights=a.out)
    print(json.dumps(rep))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
