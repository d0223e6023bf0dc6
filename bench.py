"""Throughput benchmark of the D3Q19 stream-collide path on GB300.

Workload (the channel configuration the metric is quoted on): D3Q19 MRT with
Smagorinsky LES (Cs^2 = CS = 0.01), 512x128x128 nodes, tau0 = 0.52
(RE = 3*UMAX*D/(tau0-0.5) = 120, D = 16), inlet u = 0.05 with 1 % seeded
per-node-per-step noise, zero-gradient outlet, periodic z, no-slip y walls,
a square cylinder of side 16 nodes at x = 128; the reference's momentum
exchange drag/lift is computed every step.  Synthetic inputs: the flow starts
from the equilibrium at the inlet velocity, as the reference initialises it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One JSON line on rank 0.  `value` is whole-job MLUPS with the populations
resident in HBM (N GPUs run N independent replicas: the build is single-GPU,
the metric scales weakly); `e2e` is the same run driven through the public
API from pinned host buffers (initial populations in, every step's force out,
final populations out, all inside the timed region); `roofline` is the
dominant kernel (stream-collide) against the measured HBM copy bandwidth;
`cpu_baseline` times the same workload on the host cores (the oracle's
OpenMP restatement of the channel step, about 10 s of it), and
`cpu_reference_program` the reference's own CPU program (CPU_3D/CPU_3D.cpp,
staged and built by oracle/ref_recipe.py; a lid cavity) at the same shape.
`--impl reference` times the channel step on the host cores alone (the
reference arm), with CPU_3D's figure beside it.  The default line also
carries the two-level refinement (`c3_refinement`), the closure's
training ensemble (`c5_ensemble`), the closure's data generation and
training (`c5_training`) and the FP16 / BF16 precision study at
768x256x256 over 2000 steps (`c4_precision`) on their own configurations; `--workload`
prints one of those rows, the precision study (`c4`) or the closure
deployment (`sgs`) alone.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NX, NY, NZ = 512, 128, 128
CELLS = NX * NY * NZ
BYTES_PER_CELL = {"fp32": 152, "fp16": 76, "bf16": 76, "fp64": 304}
WORKLOAD = ("D3Q19 MRT+Smagorinsky channel 512x128x128, square cylinder side 16 at x=128 with half-way "
            "bounce-back, tau0=0.52 (RE=120), CS=0.01 (Cs=0.1), inlet 0.05 + 1% seeded noise, periodic z, "
            "drag/lift every step")


SGS_WEIGHTS = ROOT / "lbm_multigpu_gb300" / "data" / "sgs_mlp.bin"
SGS_REFRESH = 16   # the refresh interval of the learned_sgs_every entry
# MLP 15(+1)->64->64->1 per cell: 2 (16*64 + 64*64 + 64) multiply-adds
SGS_FLOP_PER_CELL = 2 * (16 * 64 + 64 * 64 + 64)


def inputs_text(precision: str, tmax: int, bounceback: str = "halfway", sgs: str = "smagorinsky",
                sgs_every: int = 1) -> str:
    import lbm_multigpu_gb300 as lbm

    ext = dict(sgs="mlp", sgs_weights=str(SGS_WEIGHTS), sgs_every=sgs_every) if sgs == "mlp" else {}
    return lbm.make_inputs(NX, NY, NZ, obst1=(128.5, 63.5, 0.0), r1=8.0, re=120.0, umax=0.05, tmax=tmax, les=1,
                           cs=0.01, model="MRT", geometry="channel_square", precision=precision, inlet_noise=0.01,
                           seed=12345, bounceback=bounceback, **ext)


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return dict(hbm_gbs=float(d["hbm_gbs"]), src="measured")
    return dict(hbm_gbs=6800.0, src="fallback")


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region"""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.15)
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(name)
        return dict(sm_mhz=statistics.median(sm) if sm else None, sm_max_mhz=mx, reasons=sorted(reasons),
                    samples=len(sm))


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def time_precision(precision: str, steps: int, warmup: int, world: int, dist, with_clocks: bool, gpu: int,
                   bounceback: str = "halfway", sgs: str = "smagorinsky", keep_fields: bool = False,
                   sgs_every: int = 1):
    """resident-in-HBM run of `steps` steps after `warmup`; returns (ms, kernel ms, clocks, audit, launches,
    the final rho, u, v, w fields when keep_fields)"""
    import lbm_multigpu_gb300 as lbm

    s = lbm.Solver(inputs_text(precision, warmup + steps + 10, bounceback, sgs, sgs_every))
    s.step(warmup)
    s.synchronize()
    if dist:
        dist.barrier()
    clocks = None
    n0 = s.launch_count()
    if with_clocks:
        with ClockSampler(gpu) as cs:
            ms = s.step_timed(steps)
        clocks = cs.summary()
    else:
        ms = s.step_timed(steps)
    launches = s.launch_count() - n0
    if dist:
        dist.barrier()
    fields = s.fields() if keep_fields else None  # the state after warmup + steps steps
    audit = s.audit()
    kernel_ms = s.time_stream_collide(20)
    s.close()
    return ms, kernel_ms, clocks, audit, launches, fields


def fp64_twin_fields(nsteps: int):
    """the FP64-storage twin of the same kernels after nsteps steps (the
    accuracy reference of the reduced-precision stores), and the fluid mask"""
    import lbm_multigpu_gb300 as lbm

    with lbm.Solver(inputs_text("fp64", nsteps + 10)) as s:
        s.step(nsteps)
        return s.fields(), s.mask()


def field_errors(fields, ref, mask) -> dict:
    """max and RMS density and velocity error of fields against ref over the
    fluid nodes, and the relative L2 velocity error"""
    import numpy as np

    fl = (mask != 1) & (mask != 2)
    rho, u = fields[0][fl].astype(np.float64), np.stack([f[fl] for f in fields[1:]]).astype(np.float64)
    rr, ur = ref[0][fl].astype(np.float64), np.stack([f[fl] for f in ref[1:]]).astype(np.float64)
    dr, du = rho - rr, np.linalg.norm(u - ur, axis=0)
    return dict(rho_err_max=float(np.abs(dr).max()), rho_err_rms=float(np.sqrt(np.mean(dr ** 2))),
                u_err_max=float(du.max()), u_err_rms=float(np.sqrt(np.mean(du ** 2))),
                u_rel_l2=float(np.linalg.norm(u - ur) / np.linalg.norm(ur)))


def worst_over_ranks(ms: float, dist) -> float:
    """the slowest rank's time: the job's time for replicas run in lockstep"""
    if not dist:
        return ms
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_mlups(world: int, cells: int, steps: int, ms: float) -> float:
    """whole-job MLUPS of `world` replicas that each updated `cells` nodes
    `steps` times in `ms` (the slowest rank's time)"""
    return world * cells * steps / (ms * 1e-3) / 1e6


def time_e2e(steps: int, world: int, dist) -> dict:
    """the same workload through the public API with host buffers in the
    timed region: pinned initial populations in, each step's force out
    (queued into pinned memory, read once the loop has drained), final
    populations out"""
    import numpy as np
    import torch

    import lbm_multigpu_gb300 as lbm

    s = lbm.Solver(inputs_text("fp32", steps + 10))
    f0 = s.populations()
    host_in = torch.empty(f0.shape, dtype=torch.float32, pin_memory=True).numpy()
    host_in[...] = f0
    host_out = torch.empty(f0.shape, dtype=torch.float32, pin_memory=True).numpy()
    force = torch.zeros((steps, 3), dtype=torch.float64, pin_memory=True).numpy()
    s.init_equilibrium()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    s.set_populations(host_in)
    for i in range(steps):
        s.step(1)
        s.last_force_async(force[i])
    s.populations(out=host_out)
    s.synchronize()  # the queued force reads have landed
    t1 = time.perf_counter()
    if dist:
        dist.barrier()
    s.close()
    sec = t1 - t0
    h2d = host_in.nbytes / steps
    d2h = (host_out.nbytes + steps * 24) / steps
    return dict(sec=sec, h2d=h2d, d2h=d2h, finite=bool(np.isfinite(force).all()))


def cpu3d_binary() -> Path | None:
    for name in ("cpu3d_c2_long", "cpu3d_c2"):
        p = ROOT / "oracle" / "_ref" / name
        if p.exists() and os.access(p, os.X_OK):
            return p
    return None


def run_cpu3d(binary: Path) -> tuple[float, float]:
    """the reference CPU program at the 512x128x128 shape; its own MLUPS print"""
    r = subprocess.run([str(binary)], capture_output=True, text=True, timeout=600, cwd=str(binary.parent))
    m = re.search(r"Time taken for main kernel: ([0-9.eE+-]+) \(([0-9.eE+-]+)MLUPS\)", r.stdout)
    if not m:
        raise RuntimeError("CPU_3D did not report MLUPS: " + r.stdout[-300:] + r.stderr[-300:])
    return float(m.group(2)), float(m.group(1))


def cpu_reference_program() -> dict | None:
    """the reference's only CPU program (CPU_3D, serial, staged and built by
    oracle/ref_recipe.py) at the 512x128x128 shape: its own lid-cavity MRT,
    not the channel; None when it is not staged"""
    binary = cpu3d_binary()
    if binary is None:
        return None
    v, sec = run_cpu3d(binary)
    steps = 24 if binary.name.endswith("long") else 8
    return dict(value=v, unit="MLUPS", cores=1, kind="reference",
                sample=f"CPU_3D/CPU_3D.cpp (serial, g++ -O3), 512x128x128, {steps} steps, {sec:.1f} s of loop "
                       f"time; its lid-cavity MRT (no LES, no cylinder, no inlet) at the channel's shape")


def c2_oracle_run():
    """the oracle's restatement of the benchmarked channel step (half-way
    bounce-back, 1 % seeded inlet noise, MRT-LES, the record's mask) on all
    host cores, from the inlet-velocity equilibrium"""
    sys.path.insert(0, str(ROOT / "tests"))
    import lbm_multigpu_gb300 as lbm
    from oracle_bindings import OracleRun

    mask = lbm.inputs_mask(inputs_text("fp32", 10)).reshape(NZ, NY, NX)
    return OracleRun(NX, NY, NZ, mask, 1 / 0.52, model=0, les=1, cs=0.01, u_in=0.05, init_u=0.05, noise_amp=0.01,
                     seed=12345, halfway=1)


def timed_oracle_steps(o, steps: int, budget_s: float) -> tuple[int, float]:
    """up to `steps` oracle steps, stopping once `budget_s` seconds have
    passed; (steps done, seconds)"""
    done, t0 = 0, time.perf_counter()
    while done < steps:
        o.step(1)
        done += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    return done, time.perf_counter() - t0


def oracle_baseline(budget_s: float = 10.0) -> dict:
    """the benchmarked workload on the host cores: the oracle's OpenMP
    restatement of the channel step (pinned to the reference's own kernels),
    a bounded sample of about budget_s seconds"""
    import numpy as np

    o = c2_oracle_run()
    from oracle_bindings import oracle

    o.step(1)
    n, sec = timed_oracle_steps(o, 1000, budget_s)
    assert np.isfinite(o.fa).all()
    return dict(value=CELLS * n / sec / 1e6, unit="MLUPS", cores=int(oracle().orc_num_threads()), kind="port",
                sample=f"oracle restatement (OpenMP) of this workload, 512x128x128, {n} steps, {sec:.1f} s")


def cpu_baseline() -> dict:
    """the same workload on the host cores (the oracle port)"""
    return oracle_baseline()


def reference_arm(args, world, rank):
    """the reference arm: the benchmarked channel on the host cores.  The
    reference's own CPU program (CPU_3D) computes another case (its lid
    cavity), so the timed path is the oracle's restatement of the channel
    step, which is pinned to the reference's kernels; CPU_3D's figure at the
    same shape rides along as cpu_reference_program"""
    if rank != 0:
        return
    import numpy as np

    o = c2_oracle_run()
    from oracle_bindings import oracle

    for _ in range(max(1, min(args.warmup, 3))):
        o.step(1)
    n, sec = timed_oracle_steps(o, max(1, args.steps), 60.0)
    assert np.isfinite(o.fa).all()
    value = CELLS * n / sec / 1e6
    cores = int(oracle().orc_num_threads())
    base = dict(value=value, unit="MLUPS", cores=cores, kind="port",
                sample=f"oracle restatement (OpenMP) of this workload, 512x128x128, {n} of {args.steps} steps "
                       f"(60 s budget), {sec:.1f} s")
    line = dict(metric="MLUPS", value=value, unit="MLUPS", impl="reference", n_gpus=args.gpus, steps=n,
                warmup=args.warmup, ms_per_step=1e3 * sec / n, higher_is_better=True, scaling="weak",
                vs_baseline=None, dtype="f32", data="synthetic (equilibrium start at the inlet velocity, seeded "
                                                    "inlet noise)",
                config=dict(workload=WORKLOAD, same_config=True,
                            note="the channel step on all host cores; the reference's own CPU program (CPU_3D) "
                                 "computes a lid cavity and is reported beside it"),
                cpu_baseline=base, e2e=dict(value=value, unit="MLUPS", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    prog = cpu_reference_program()
    if prog is not None:
        line["cpu_reference_program"] = prog
    print(json.dumps(line))


C3_PATCH = dict(lr_dims=(96, 64, 64), lr_origin=(48.25, 47.25, 16.25), cf_time="linear")


def c3_inputs(tmax: int, lr_dims=C3_PATCH["lr_dims"], lr_origin=C3_PATCH["lr_origin"],
              cf_time=C3_PATCH["cf_time"]) -> str:
    """the two-level refinement record: coarse 256x128x64 MRT-LES channel,
    circular cylinder of diameter 12 coarse cells at (64.5, 63.5), ratio-2
    patch (by default the configured 96x64x64 fine cells bounded in z from
    coarse z 16.25, linear temporal interpolation), tau0 = 0.52, 1 % noise"""
    import lbm_multigpu_gb300 as lbm

    return lbm.make_inputs(256, 128, 64, obst1=(64.5, 63.5, 0.0), r1=6.0, re=90.0, umax=0.05, tmax=tmax, les=1,
                           cs=0.01, geometry="channel_circle", refinement=1, lr_dims=lr_dims, lr_factor=0.5,
                           lr_origin=lr_origin, inlet_noise=0.01, cf_time=cf_time)


def workload_c3(steps: int, warmup: int) -> dict:
    """two-level refinement as the configuration names it: coarse 256x128x64
    MRT-LES channel, circular cylinder of diameter 12 coarse cells, a ratio-2
    fine patch of 96x64x64 fine cells (bounded in z: coarse planes 16-48),
    second-order spatial and linear temporal coarse-to-fine interpolation,
    2 fine steps per coarse step; MLUPS by the reference's count
    (LR7:2956-2961): coarse nodes + fine nodes x LRLEVEL per coarse step.
    Beside it the reference's own layout (patch spanning the periodic z
    extent, 96x64x128, no time interpolation)."""
    import lbm_multigpu_gb300 as lbm

    def run(lr_dims, lr_origin, cf_time):
        text = c3_inputs(steps + warmup + 10, lr_dims, lr_origin, cf_time)
        with lbm.Solver(text) as s:
            s.step(warmup)
            s.synchronize()
            n0 = s.launch_count()
            ms = s.step_timed(steps)
            launches = s.launch_count() - n0
            kc = s.time_stream_collide(20, 0)
            kf = s.time_stream_collide(20, 1)
            audit = s.audit(0)
        nodes = 256 * 128 * 64 + lr_dims[0] * lr_dims[1] * lr_dims[2] * 2
        return dict(value=nodes * steps / (ms * 1e3), ms_per_coarse_step=ms / steps,
                    kernel_ms=dict(coarse_stream_collide=kc, fine_stream_collide=kf,
                                   interface_and_force=ms / steps - kc - 2 * kf),
                    gpu_launches=launches, audit_mass=float(audit[0]))

    main = run(C3_PATCH["lr_dims"], C3_PATCH["lr_origin"], C3_PATCH["cf_time"])
    ref = run((96, 64, 128), (48.25, 47.25, -0.75), "none")
    return dict(workload="C3 two-level refinement: coarse 256x128x64 + fine 96x64x64 (ratio 2, bounded in z from "
                         "coarse z 16.25), linear temporal interpolation, MRT-LES, circular cylinder D=12, tau0=0.52 "
                         "(RE=90), CS=0.01, 1% inlet noise",
                metric="MLUPS (coarse + 2 x fine nodes per coarse step)", unit="MLUPS", steps=steps, warmup=warmup,
                **main,
                reference_layout=dict(ref, note="fine 96x64x128 spanning the periodic z extent, no time "
                                                "interpolation (LR7's layout and schedule)"))


def workload_c4(steps: int, every: int = 250) -> dict:
    """precision: the channel geometry scaled to 768x256x256 (square cylinder
    side 24 at x=192, tau0=0.52) with populations stored as FP16 / BF16
    (deviations from the MRT equilibrium at (1, u_in)), FP32 collide, beside
    FP32 and an FP64-storage twin of the same kernels, advanced side by side:
    max / RMS density and velocity error of each against FP64 every `every`
    steps (the error-vs-step trace), and MLUPS from the summed step times"""
    import numpy as np

    import lbm_multigpu_gb300 as lbm

    nx, ny, nz = 768, 256, 256
    precs = ("fp64", "fp32", "fp16", "bf16")
    solvers = {}
    for prec in precs:
        solvers[prec] = lbm.Solver(lbm.make_inputs(nx, ny, nz, obst1=(192.5, 127.5, 0.0), r1=12.0, re=180.0,
                                                   umax=0.05, tmax=steps + 10, les=1, cs=0.01,
                                                   geometry="channel_square", precision=prec, bounceback="halfway"))
    mask = solvers["fp64"].mask()
    ms = {prec: 0.0 for prec in precs}
    trace = {prec: [] for prec in precs[1:]}
    done = 0
    while done < steps:
        k = min(every, steps - done)
        for prec in precs:
            ms[prec] += solvers[prec].step_timed(k)
        done += k
        ref = solvers["fp64"].fields()
        for prec in precs[1:]:
            e = field_errors(solvers[prec].fields(), ref, mask)
            trace[prec].append(dict(step=done, **e))
    for s_ in solvers.values():
        s_.close()
    out = {}
    for prec in precs:
        out[prec] = dict(mlups=nx * ny * nz * steps / (ms[prec] * 1e3), ms_per_step=ms[prec] / steps)
        if prec != "fp64":
            out[prec].update({k: v for k, v in trace[prec][-1].items() if k != "step"})
            out[prec]["trace"] = [dict(step=t["step"], u_rel_l2=t["u_rel_l2"], u_err_rms=t["u_err_rms"],
                                       rho_err_rms=t["rho_err_rms"]) for t in trace[prec]]
    for prec in ("fp16", "bf16"):
        out[prec]["mlups_vs_fp32"] = out[prec]["mlups"] / out["fp32"]["mlups"]
    return dict(workload="C4 precision: 768x256x256 channel, square cylinder side 24, MRT-LES, half-way "
                         "bounce-back; errors over fluid nodes against the FP64-storage twin, traced every "
                         f"{every} steps",
                steps=steps, results=out)


def workload_sgs_channel(steps: int, warmup: int) -> dict:
    """the learned closure deployed in the channel: MLUPS of the tensor-core
    MLP stream-collide against Smagorinsky on the same 512x128x128 case"""
    import lbm_multigpu_gb300 as lbm

    res = {}
    for name, sgs, every in (("smagorinsky", "smagorinsky", 1), ("mlp", "mlp", 1),
                             (f"mlp_every{SGS_REFRESH}", "mlp", SGS_REFRESH)):
        with lbm.Solver(inputs_text("fp32", steps + warmup + 10, sgs=sgs, sgs_every=every)) as s:
            s.step(warmup)
            ms = s.step_timed(steps)
            k = s.time_stream_collide(20)
        res[name] = dict(mlups=CELLS * steps / (ms * 1e3), ms_per_step=ms / steps, kernel_ms=k)
    res["cost"] = 1 - res["mlp"]["mlups"] / res["smagorinsky"]["mlups"]
    res[f"cost_every{SGS_REFRESH}"] = 1 - res[f"mlp_every{SGS_REFRESH}"]["mlups"] / res["smagorinsky"]["mlups"]
    res["tensor_tflops"] = CELLS * SGS_FLOP_PER_CELL / (res["mlp"]["kernel_ms"] * 1e-3) / 1e12
    return dict(workload="C5 deployment: " + WORKLOAD.replace("MRT+Smagorinsky", "MRT + learned closure"),
                steps=steps, results=res)


def workload_ensemble(steps: int, warmup: int) -> dict:
    """C5 batching: the 16-member decaying-turbulence ensemble of uneven box
    sizes (64^3..160^3, seeded) advanced by one persistent launch per step
    from a CUDA graph, tile height and grid from the autotuner; MRT, periodic;
    MLUPS over all members and the fraction of the HBM roofline (152 B per
    node update)"""
    import lbm_multigpu_gb300 as lbm
    from lbm_multigpu_gb300 import sgs_pipeline as sp

    sizes = sp.ensemble_sizes(2024, 16)
    with lbm.Ensemble(sizes, sp.TAU_F, sgs="none") as e:
        e.init_turbulence(2024, kmax_div=8, per_shell=24)
        ty, grid, tuned = e.autotune()
        e.step(warmup)
        ms = e.step_timed(steps)
        cells = e.info()["cells"]
    gbs = cells * 152 / (ms / steps * 1e-3) / 1e9
    pk = peaks()
    return dict(workload="C5 ensemble: 16 periodic MRT boxes, sides " + ",".join(map(str, sizes)),
                metric="MLUPS", value=cells * steps / (ms * 1e3), unit="MLUPS", steps=steps, cells=cells,
                ms_per_step=ms / steps, tile=f"32x{ty}", grid=grid, autotune_ms_per_step=tuned,
                roofline=dict(bound="hbm", achieved=gbs, peak=pk["hbm_gbs"], unit="GB/s", frac=gbs / pk["hbm_gbs"]))


def workload_training(train_steps: int = 1000) -> dict:
    """C5 training: the 16-member ensemble at 2x resolution advanced and
    box-filtered into samples (lbm_multigpu_gb300.sgs_pipeline.generate),
    then train_steps Adam steps of the fused forward/backward kernels on
    them (batch 16384, the closure's coefficient targets)"""
    import torch

    from lbm_multigpu_gb300 import sgs_pipeline as sp

    sizes = sp.ensemble_sizes(2024, 16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    X, T, gen = sp.generate(sizes, 2024)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    T = sp.coefficient_targets(X, T)
    P, hist, t_train = sp.train(X, T, steps=train_steps)
    return dict(workload="C5 training: 16-box ensemble (" + ",".join(map(str, sizes)) + ") at 2x, 6 snapshots, "
                         f"{train_steps} Adam steps of batch 16384",
                samples=int(X.shape[0]), ensemble_fine_steps=gen["fine_steps"], ensemble_mlups=gen["mlups"],
                generate_s=t_gen, train_steps=train_steps, train_s=t_train,
                train_samples_per_s=train_steps * 16384 / t_train, loss_first=float(hist[:10].mean()),
                loss_last=float(hist[-10:].mean()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--precision", default="all", choices=["all", "fp32", "fp16", "bf16"],
                    help="storage precisions to time (all: fp32 reference point, then fp16 and bf16)")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "sgs", "ensemble"],
                    help="c2: the channel headline line (default); c3: two-level refinement; c4: storage "
                         "precision against FP64 at 768x256x256; sgs: the learned closure against Smagorinsky; "
                         "ensemble: the 16-member periodic-box ensemble")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()

    if args.impl == "reference":
        reference_arm(args, world, rank)
        return

    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as td

        td.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = td
    import __graft_entry__

    if rank == 0 or not (ROOT / "lbm_multigpu_gb300" / "_build" / "liblbm_gb300.so").exists():
        __graft_entry__.build()
    if args.workload != "c2":
        if rank == 0:
            steps = min(args.steps, 2000)
            if args.workload == "c3":
                line = workload_c3(steps, args.warmup)
            elif args.workload == "c4":
                line = workload_c4(steps)
            elif args.workload == "ensemble":
                line = workload_ensemble(steps, args.warmup)
            else:
                line = workload_sgs_channel(steps, args.warmup)
            print(json.dumps(line))
        return
    if dist:
        dist.barrier()
    import numpy as np

    # FP32 Smagorinsky (the reference point), then the FP16 / BF16 stores
    main_prec = "fp32" if args.precision == "all" else args.precision
    ms32, kms32, clocks, audit, launches, f32 = time_precision(main_prec, args.steps, args.warmup, world, dist, True,
                                                               local, keep_fields=True)
    res, fields = {}, {main_prec: f32}
    for prec in (("fp16", "bf16") if args.precision == "all" else ()):
        ms, kms, _, _, _, fields[prec] = time_precision(prec, args.steps, args.warmup, world, dist, False, local,
                                                       keep_fields=True)
        res[prec] = (ms, kms)
    full = sgsr = None
    if args.precision == "all" and SGS_WEIGHTS.exists():
        # the learned closure in place of Smagorinsky (tensor-core MLP per tile)
        mss, kmss, _, _, _, _ = time_precision("fp32", args.steps, args.warmup, world, dist, False, local, sgs="mlp")
        sgsr = (mss, kmss)
        # the same closure evaluated every SGS_REFRESH steps, its eddy
        # viscosity reused per node in between, timed over whole refresh
        # periods (every window of k steps holds one refresh)
        nref = SGS_REFRESH * max(1, -(-args.steps // SGS_REFRESH))
        msr, _, _, _, _, _ = time_precision("fp32", nref, args.warmup, world, dist, False, local, sgs="mlp",
                                            sgs_every=SGS_REFRESH)
        sgsr = (mss, kmss, msr, nref)
    if args.precision == "all":
        # the reference's own wall treatment (full-way, on-node bounce-back)
        msf, kmsf, _, _, _, _ = time_precision("fp32", args.steps, args.warmup, world, dist, False, local, "fullway")
        full = (msf, kmsf)
    # every storage precision against the FP64 twin of the same steps
    acc = {}
    if rank == 0:
        ref, mask = fp64_twin_fields(args.warmup + args.steps)
        acc = {prec: field_errors(f, ref, mask) for prec, f in fields.items()}

    def worst(ms):
        return worst_over_ranks(ms, dist)

    ms32 = worst(ms32)
    for prec in res:
        res[prec] = (worst(res[prec][0]), res[prec][1])
    e2e = None if args.no_e2e else time_e2e(min(args.steps, 2000), world, dist)
    e2e_sec = worst(e2e["sec"]) if e2e else None

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    pk = peaks()
    mlups = replica_mlups(world, CELLS, args.steps, ms32)
    kernel_gbs = CELLS * BYTES_PER_CELL[main_prec] / (kms32 * 1e-3) / 1e9
    traffic = None
    prof = ROOT / "profiles" / "traffic.json"
    if prof.exists():
        traffic = json.loads(prof.read_text()).get(f"k_stream_collide<{main_prec}>")
    line = dict(
        metric="MLUPS", value=mlups, unit="MLUPS", n_gpus=world, steps=args.steps, warmup=args.warmup,
        ms_per_step=ms32 / args.steps, higher_is_better=True, scaling="weak", vs_baseline=None,
        dtype={"fp32": "f32", "fp16": "f16 storage, f32 math", "bf16": "bf16 storage, f32 math"}[main_prec],
        data="synthetic (equilibrium start at the inlet velocity, seeded Philox inlet noise)",
        config=dict(workload=WORKLOAD, parallelism="replicas only" if world > 1 else "single GPU",
                    cache="inputs >= 0.64 GB per step > 129 MB L2: no flush needed",
                    precision=f"{main_prec} storage, fp32 math",
                    forces="FP64 momentum exchange every step"),
        roofline=dict(bound="hbm", achieved=kernel_gbs, peak=pk["hbm_gbs"], unit="GB/s",
                      frac=kernel_gbs / pk["hbm_gbs"], traffic=traffic,
                      peak_src=f"{pk['src']} (MEASURED_PEAKS.json hbm_gbs, burst copy)",
                      kernel=f"k_stream_collide<{main_prec}>", kernel_ms=kms32,
                      algorithmic_bytes_per_cell=BYTES_PER_CELL[main_prec]),
        e2e=None if not e2e else dict(value=world * CELLS * min(args.steps, 2000) / e2e_sec / 1e6, unit="MLUPS",
                                      h2d_bytes_per_step=e2e["h2d"], d2h_bytes_per_step=e2e["d2h"],
                                      steps=min(args.steps, 2000)),
        gpu_launches=launches * world,
        accuracy_vs_fp64=dict(acc.get(main_prec, {}), steps=args.warmup + args.steps),
        clocks=clocks,
        audit=dict(mass=float(audit[0]), momentum=[float(a) for a in audit[1:]]),
    )
    for prec, (ms, kms) in res.items():
        v = world * CELLS * args.steps / (ms * 1e-3) / 1e6
        gbs = CELLS * BYTES_PER_CELL[prec] / (kms * 1e-3) / 1e9
        line[f"{prec}_store"] = dict(value=v, ratio_vs_fp32=v / mlups, ms_per_step=ms / args.steps,
                                     kernel_ms=kms, kernel_gbs=gbs, frac=gbs / pk["hbm_gbs"],
                                     accuracy_vs_fp64=dict(acc.get(prec, {}), steps=args.warmup + args.steps))
    if full:
        v = world * CELLS * args.steps / (worst(full[0]) * 1e-3) / 1e6
        gbs = CELLS * BYTES_PER_CELL["fp32"] / (full[1] * 1e-3) / 1e9
        line["fp32_fullway_bounceback"] = dict(value=v, ms_per_step=worst(full[0]) / args.steps, kernel_ms=full[1],
                                               kernel_gbs=gbs, frac=gbs / pk["hbm_gbs"])
    if sgsr:
        v = world * CELLS * args.steps / (worst(sgsr[0]) * 1e-3) / 1e6
        gbs = CELLS * BYTES_PER_CELL["fp32"] / (sgsr[1] * 1e-3) / 1e9
        line["learned_sgs"] = dict(value=v, ratio_vs_smagorinsky=v / mlups, cost=1 - v / mlups,
                                   ms_per_step=worst(sgsr[0]) / args.steps, kernel_ms=sgsr[1], kernel_gbs=gbs,
                                   frac=gbs / pk["hbm_gbs"],
                                   tensor_tflops=CELLS * SGS_FLOP_PER_CELL / (sgsr[1] * 1e-3) / 1e12,
                                   kernel="k_stream_collide_mlp<fp32>", weights=str(SGS_WEIGHTS.relative_to(ROOT)))
        vr = world * CELLS * sgsr[3] / (worst(sgsr[2]) * 1e-3) / 1e6
        line[f"learned_sgs_every{SGS_REFRESH}"] = dict(
            value=vr, ratio_vs_smagorinsky=vr / mlups, cost=1 - vr / mlups, ms_per_step=worst(sgsr[2]) / sgsr[3],
            steps=sgsr[3],
            note=f"SGS every: {SGS_REFRESH} -- the closure's kernel on the steps t % {SGS_REFRESH} == 0, its "
                 "per-node eddy viscosity reused by the plain stream-collide in between")
    if args.precision == "all":
        # the other GPU rows of the scope, each on its own configuration
        # (rank 0, after the timed region): two-level refinement as configured
        # and the closure's training ensemble
        line["c3_refinement"] = workload_c3(min(args.steps, 500), max(args.warmup, 3))
        line["c5_ensemble"] = workload_ensemble(min(args.steps, 64), max(args.warmup, 3))
        # the precision study at its configured 2000 steps, errors at the end
        line["c4_precision"] = workload_c4(2000, every=2000)
        line["c5_training"] = workload_training()
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
        prog = cpu_reference_program()
        if prog is not None:
            line["cpu_reference_program"] = prog
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
