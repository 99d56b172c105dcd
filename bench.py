#!/usr/bin/env python
"""Monostatic RCS sweep benchmark on GB300 (angle.pol/s).

Default workload (the precision configuration of the benchmark set): PEC
tangent cone-sphere, hemisphere a = 0.5 m, 15 deg half-angle, ka = 40 (k = 80),
N = 1200 equal-arc segments, |m| <= 50, 361 aspect angles (0.5 deg steps) x
2 polarisations = 722 angle.pol per sweep.  A "step" is one complete sweep:
far fill, FP64 near/self fill, LU of every mode, solves, FP64 refinement,
far-field mode sum.

  value   722 * ranks / device seconds per step, FP32+IR path, geometry tables
          already resident in HBM
  e2e     the same metric through the public drop-in API solve_bor() with host
          (NumPy) inputs: host set-up, host->device table copies, device->host
          results inside the timed region
  fp64_plain   the same sweep through the plain FP64 GPU path (comparator)

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun each rank runs an independent replica (weak scaling).
"""

from __future__ import annotations

import argparse
import csv
import importlib
import io
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
PKG = "20260722_ghost_gb300"
C0 = 299_792_458.0

WORKLOADS = {
    "cone_sphere_ka40": dict(body="cone_sphere", a=0.5, half_angle=15.0, N=1200, k=80.0, M=50,
                             dtheta=0.5),
    "sphere_ka10": dict(body="sphere", a=1.0, N=240, k=10.0, M=20, dtheta=1.0),
    # profiling size: same body at half the frequency, ~2 GB on the device
    "cone_sphere_ka20": dict(body="cone_sphere", a=0.5, half_angle=15.0, N=600, k=40.0, M=25,
                             dtheta=0.5),
    "cone_sphere_ka100": dict(body="cone_sphere", a=0.5, half_angle=15.0, N=3000, k=200.0, M=120,
                              dtheta=0.25),
    # clamped cubic B-spline body, 64 control radii r_j ~ U(0.3, 0.6) (numpy seed 0)
    # on a 2 m axis, ka = 20 at r = 0.5; objective mean sigma_HH over 30..60 deg;
    # the line adds the adjoint gradient leg
    # 64 seeded random bodies (bodies.random_bodies, seed 0): N ~ U{200..1600},
    # 12 segments per wavelength, |m| <= ceil(k rho_max) + 10, 181 angles x 2 pols
    "random64": dict(body="random", n_bodies=64, N=0, k=0.0, M=0, dtheta=1.0),
    "bspline_ka20": dict(body="bspline", n_radii=64, N=600, k=40.0, M=30, theta0=30.0, theta1=60.0,
                         dtheta=0.5, pol="HH"),
}
METRIC = "monostatic RCS angle·pol/s on 1 GB300: FP32+IR batched vs FP64 plain, ≤0.01 dB err"


def workload_inputs(name):
    import numpy as np
    w = WORKLOADS[name]
    bodies = importlib.import_module(PKG + ".bodies")
    if w["body"] == "random":
        # the CPU baseline of the batch samples its first body
        b = bodies.random_bodies(w["n_bodies"], 0)[0]
        return b["points"], b["freq_hz"], np.arange(0.0, 180.0 + 1e-9, w["dtheta"]), b["m_max"]
    if w["body"] == "sphere":
        pts = bodies.sphere_generatrix(w["a"], w["N"])
    elif w["body"] == "bspline":
        pts = bodies.bspline_body(bspline_radii(w), w["N"])[0]
    else:
        pts = bodies.cone_sphere_generatrix(w["a"], w["half_angle"], w["N"])
    thetas = np.arange(w.get("theta0", 0.0), w.get("theta1", 180.0) + 1e-9, w["dtheta"])
    return pts, w["k"] * C0 / (2 * math.pi), thetas, w["M"]


def bspline_radii(w):
    import numpy as np
    return np.random.default_rng(0).uniform(0.3, 0.6, w["n_radii"])


def adjoint_leg(w, f, thetas):
    """Adjoint gradient of mean sigma_pol w.r.t. the control radii: timing of
    the forward sweep and the backward pass, FP32+IR vs FP64 gradient, and
    central differences (h = 1e-4 m, FP64 solves) on four radii."""
    import numpy as np
    import torch
    adj = importlib.import_module(PKG + ".adjoint")
    r = bspline_radii(w)
    pol = w["pol"]
    adj.bspline_rcs_and_gradient(r, w["N"], f, thetas, pol, w["M"], "fp32ir")        # warm-up
    tm = {}
    J32, g32 = adj.bspline_rcs_and_gradient(r, w["N"], f, thetas, pol, w["M"], "fp32ir", timings=tm)
    tm64 = {}
    J64, g64 = adj.bspline_rcs_and_gradient(r, w["N"], f, thetas, pol, w["M"], "fp64", timings=tm64)
    h = 1e-4
    checks = []

    def central(j, hh):
        Js = []
        for sgn in (1.0, -1.0):
            rr = r.copy()
            rr[j] += sgn * hh
            Js.append(adj.objective(adj._bspline_forward(rr, w["N"], f, thetas, pol, w["M"], "fp64", 1.0)[2],
                                    pol))
        return (Js[0] - Js[1]) / (2 * hh)

    for j in (0, len(r) // 3, 2 * len(r) // 3, len(r) - 1):
        fd = central(j, h)
        # Richardson extrapolation of the central difference (h, h/2) removes
        # its O(h^2) truncation error, which is large for this objective
        fd_r = (4.0 * central(j, h / 2) - fd) / 3.0
        den = max(abs(fd_r), 1e-3 * float(np.max(np.abs(g64))))
        checks.append({"param": j, "fd": fd, "fd_richardson": fd_r, "adjoint_fp32ir": float(g32[j]),
                       "adjoint_fp64": float(g64[j]), "rel_err_fp32ir": abs(g32[j] - fd_r) / den,
                       "rel_err_fp64": abs(g64[j] - fd_r) / den, "rel_err_fp32ir_plain_fd": abs(g32[j] - fd) / den})
    torch.cuda.synchronize()
    return {"objective": f"mean sigma_{pol} over {thetas[0]:g}..{thetas[-1]:g} deg (m^2)", "J_fp32ir": J32,
            "J_fp64": J64, "n_params": len(r), "forward_s": tm["forward_s"], "gradient_s": tm["gradient_s"],
            "forward_fp64_s": tm64["forward_s"], "gradient_fp64_s": tm64["gradient_s"],
            "grad_fp32ir_vs_fp64_rel": float(np.max(np.abs(g32 - g64)) / np.max(np.abs(g64))),
            "fd_check": {"h": h, "method": "central differences of FP64 solves at h and h/2, Richardson-"
                                            "extrapolated; rel_err_*_plain_fd: against the plain h = 1e-4 value",
                         "max_rel_err_fp32ir": max(c["rel_err_fp32ir"] for c in checks),
                         "max_rel_err_fp64": max(c["rel_err_fp64"] for c in checks),
                         "max_rel_err_fp32ir_plain_fd": max(c["rel_err_fp32ir_plain_fd"] for c in checks),
                         "params": checks}}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms in the background."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r for r in csv.reader(open(self.path)) if len(r) >= 9]
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if "Active" in v and "Not" not in v})
        loaded = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows)}


def load_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d.get("hbm_gbs"), "bf16_tflops": d.get("bf16_tflops"), "sm_max_mhz": d.get("sm_max_mhz"),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def max_over_ranks(x: float) -> float:
    """Maximum of a per-rank time over the process group (one value per rank);
    works on the nccl (CUDA tensor) and gloo (CPU tensor) backends."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, seconds: float) -> float:
    """Whole-job throughput of independent replicas: every rank processes
    units_per_rank; the job takes the slowest rank's time."""
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    return units_per_rank * world / max_over_ranks(seconds)


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port of the reference algorithm on the host cores
# ---------------------------------------------------------------------------

_CPU_SOLVERS = {}     # workload -> oracle solver with its complete near cache


def cpu_baseline(workload: str, cores: int):
    """Time a bounded sample of the reference algorithm (the oracle port) and
    extrapolate to the full sweep: a slice of the far-field sweep, a subset of
    near element pairs and one |m| (both signs) with every angle/polarisation.
    Returns (angle.pol/s, sample description, seconds spent)."""
    import numpy as np
    from oracle import build_oracle
    build_oracle.build()
    from oracle import bor_oracle as O
    pts, f, thetas, M = workload_inputs(workload)
    t_start = time.perf_counter()
    s = O.OracleSolver(pts, f)
    ne = s.geo.ne
    n_far = min(ne, 2 * cores)
    t0 = time.perf_counter()
    s.build_far(M, efie=True, workers=cores, elem_range=(0, n_far))
    t_far = (time.perf_counter() - t0) * ne / n_far
    pairs = s.near_pairs()
    sub = pairs[:: max(1, len(pairs) // (8 * cores))]
    t0 = time.perf_counter()
    s.prepare(M, efie=True, workers=cores, pairs=sub)
    t_near = (time.perf_counter() - t0) * len(pairs) / len(sub)
    # one |m|: the complete near cache is needed by assemble; the rest is filled
    # untimed once per workload and kept for later calls (the reference arm's
    # steps), whose far and near samples above are still computed afresh
    if workload in _CPU_SOLVERS:
        s = _CPU_SOLVERS[workload]
    else:
        s.prepare(M, efie=True, workers=cores, pairs=[p for p in pairs if p not in set(sub)])
        _CPU_SOLVERS[workload] = s
    am = max(1, M // 2)
    t0 = time.perf_counter()
    for m in (am, -am):
        Z = s.assemble_efie(m, M)
        mask = s.basis_mask(m)
        V = np.stack([s.rhs_efie(m, thetas, "VV"), s.rhs_efie(m, thetas, "HH")], axis=1)
        Bm = V.transpose(2, 0, 1).reshape(2 * s.geo.Nn, -1)[mask]
        X = np.linalg.solve(Z[np.ix_(mask, mask)], Bm)
        full = np.zeros((2 * s.geo.Nn, X.shape[1]), complex)
        full[mask] = X
        xs = full.T.reshape(len(thetas), 2, -1)
        s.farfield(m, xs[:, 0, :], thetas)
        s.farfield(m, xs[:, 1, :], thetas)
    t_mode = (time.perf_counter() - t0) / 2.0
    total = t_far + t_near + t_mode * (2 * M + 1)
    sampled = t_far * n_far / ne + t_near * len(sub) / len(pairs) + 2.0 * t_mode
    sample = (f"oracle port of the reference sweep on {cores} host threads: far sweep over "
              f"{n_far}/{ne} test elements, {len(sub)}/{len(pairs)} near element pairs, one |m| "
              f"(m=+-{am}) solved for all {2 * len(thetas)} columns ({sampled:.1f} s timed), scaled by "
              f"element pairs and mode systems to the whole sweep ({total:.0f} s, x{total / sampled:.0f})")
    return 2 * len(thetas) / total, sample, time.perf_counter() - t_start, sampled, total


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_gpu(args, rank, world):
    import numpy as np
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    eng = importlib.import_module(PKG + ".engine")
    bs = importlib.import_module(PKG + ".bor_solver")
    nat = importlib.import_module(PKG + "._native")
    pts, f, thetas, M = workload_inputs(args.workload)
    prob = eng.BorGpuProblem(pts, f, thetas, m_max=M)
    angle_pol = 2 * len(thetas)
    dist = world > 1

    def barrier():
        if dist:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        prob.sweep("fp32ir")
    torch.cuda.synchronize()
    barrier()
    stages = {}
    l0 = nat.launch_count()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        torch.cuda.synchronize()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        results = []
        kernel_s, kernel_w = {}, {}
        for _ in range(args.steps):
            r = prob.sweep("fp32ir")
            results.append(r)
            for kk, v in r.timings.items():
                stages[kk] = stages.get(kk, 0.0) + v / args.steps
            for kk, v in r.kernel_s.items():
                kernel_s.setdefault(kk, []).extend(v)
                kernel_w.setdefault(kk, []).extend([kernel_work(prob, kk)] * len(v))
        e1.record()
        torch.cuda.synchronize()
        barrier()
    launches = nat.launch_count() - l0
    dev_s = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps)
    value = replica_throughput(angle_pol, dev_s)
    clocks = clk.summary()

    # FP64 plain comparator (same sweep, FP64 fill/LU/solve/residual); its
    # warm-up sweep is skipped when one FP32+IR sweep already takes > 5 s
    if dev_s < 5.0:
        r64 = prob.sweep("fp64")
        torch.cuda.synchronize()
    f64_steps = max(1, args.steps // 3)
    e0.record()
    for _ in range(f64_steps):
        r64 = prob.sweep("fp64")
    e1.record()
    torch.cuda.synchronize()
    f64_s = e0.elapsed_time(e1) / 1e3 / f64_steps
    F32 = results[-1].dF.sum(0)
    F64 = r64.dF.sum(0)
    vs_ref = accuracy_vs_reference(args.workload, thetas, F32, F64)
    db = float(np.max(np.abs(20 * np.log10(np.abs(F32) / np.abs(F64)))))
    rel = float(np.max(np.abs(F32 - F64)) / np.max(np.abs(F64)))
    acc_extra = db_stats(F32, F64)

    # end to end through the public API with host inputs
    bs.solve_bor(pts, f, thetas, n_modes=M, mode_tol=0.0, table_precision="auto")
    torch.cuda.synchronize()
    barrier()
    e2e_steps = max(1, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        out = bs.solve_bor(pts, f, thetas, n_modes=M, mode_tol=0.0, table_precision="auto")
    torch.cuda.synchronize()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps)
    h2d = prob.h2d_bytes()
    d2h = (M + 1) * angle_pol * 16 + (M + 1) * (2 * 8 + 4)
    adjoint = adjoint_leg(WORKLOADS[args.workload], f, thetas) if WORKLOADS[args.workload]["body"] == "bspline" \
        else None
    return dict(adjoint=adjoint, vs_ref=vs_ref, value=value, dev_s=dev_s, stages=stages, kernel_s=kernel_s,
                kernel_work=kernel_w, steps=args.steps, clocks=clocks, launches=launches,
                f64_s=f64_s, f64_steps=f64_steps, db=db, rel=rel, acc_extra=acc_extra, e2e_s=e2e_s, h2d=h2d, d2h=d2h,
                refine_iters=results[-1].refine_iters, residual=float(np.max(results[-1].residual)),
                prob=prob, angle_pol=angle_pol, M=M, thetas=thetas)


# amplitudes of the reference's own FP64 solve_bor, stored by
# tests/golden/make_fullsize_golden.py (the reference cannot run here)
REFERENCE_FIXTURES = {"cone_sphere_ka40": "c2_conesphere_ref.npz"}


def accuracy_vs_reference(workload, thetas, F32, F64):
    """Max relative amplitude and dB errors of the FP32+IR and the FP64 sweeps
    against the reference's FP64 amplitudes, where a fixture exists."""
    import numpy as np
    name = REFERENCE_FIXTURES.get(workload)
    path = os.path.join(HERE, "tests", "golden", name) if name else None
    if not path or not os.path.exists(path):
        return None
    D = np.load(path)
    if D["thetas"].shape != thetas.shape or not np.allclose(D["thetas"], thetas):
        return None
    ref = np.stack([D["amp_vv"], D["amp_hh"]])
    out = {"fixture": f"tests/golden/{name}", "reference_wall_s": float(D["wall_s"]),
           "reference_cores": int(D["host_cores"])}
    for tag, F in (("fp32ir", F32), ("fp64", F64)):
        out[f"{tag}_max_rel_amp_err"] = float(np.max(np.abs(F - ref)) / np.max(np.abs(ref)))
        out[f"{tag}_max_db_err"] = float(np.max(np.abs(20 * np.log10(np.abs(F) / np.abs(ref)))))
    return out


def db_stats(F32, F64):
    """dB error statistics of the FP32+IR far field against FP64 over every
    angle and polarisation: percentiles, the maximum over angles within 60 dB
    of the peak of their polarisation, and the depth of the worst angle."""
    import numpy as np
    a64 = np.abs(F64)
    db = np.abs(20 * np.log10(np.abs(F32) / a64))
    depth = 20 * np.log10(a64 / a64.max(axis=1, keepdims=True))
    i = np.unravel_index(np.argmax(db), db.shape)
    return {"db_err_p50": float(np.percentile(db, 50)), "db_err_p99": float(np.percentile(db, 99)),
            "max_db_err_within_60db_of_peak": float(np.max(db[depth > -60.0])),
            "depth_db_at_max_err": float(depth[i])}


def kernel_work(prob, name):
    """Algorithmic flops of one launch (complex MAC = 8 real flops)."""
    import numpy as np
    n, M1, nrhs = prob.n, prob.m_max + 1, prob.nrhs
    if name in ("residual", "residual_update"):
        return 8.0 * n * n * nrhs * M1
    if name == "far_fill":
        # DCT of every far Gauss-point pair: (n_xi/2 + 1) samples x (M + 2)
        # orders x complex-by-real multiply-add (4 flops)
        P = 4 * prob.N
        return 4.0 * P * P * (prob.n_xi // 2 + 1) * (prob.m_max + 2)
    # near fill: cos(m xi) projection of every near point pair, (48 + n_tail)
    # azimuth nodes x (M + 2) orders x 4 flops
    cnt = prob.near.pairs[:, 3].astype(float)
    nodes = 48.0 + prob.near.tails[:, 1].astype(float)
    return 4.0 * float(np.sum(cnt * nodes)) * (prob.m_max + 2)


def run_batch(args, rank, world):
    """Batch workload: the 64 seeded bodies as size classes (batch.BorGpuBatch:
    one LU / substitution / refinement for all modes of the bodies of a class;
    classes stream through memory when the batch does not fit), the same bodies
    back to back through the single-body sweep, the public solve_bor_batch with
    host inputs (e2e), and FP64 plain on every 16th body."""
    import numpy as np
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    eng = importlib.import_module(PKG + ".engine")
    bs = importlib.import_module(PKG + ".bor_solver")
    nat = importlib.import_module(PKG + "._native")
    bmod = importlib.import_module(PKG + ".batch")
    w = WORKLOADS[args.workload]
    bodies = importlib.import_module(PKG + ".bodies").random_bodies(w["n_bodies"], 0)
    thetas = np.arange(0.0, 180.0 + 1e-9, w["dtheta"])
    probs = [eng.BorGpuProblem(b["points"], b["freq_hz"], thetas, m_max=b["m_max"]) for b in bodies]
    angle_pol = 2 * len(thetas) * len(bodies)
    batch = bmod.BorGpuBatch(probs, tuner=bmod.Autotuner())

    for _ in range(args.warmup):
        batch.sweep()
    torch.cuda.synchronize()
    l0 = nat.launch_count()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        last = []
        for _ in range(args.steps):
            last = batch.sweep()
        e1.record()
        torch.cuda.synchronize()
    launches = nat.launch_count() - l0
    if batch.resident():            # graph replays launch no library kernel from the host
        launches = args.steps * sum(c.launches for c in batch.classes)
    dev_s = max_over_ranks(e0.elapsed_time(e1) / 1e3 / args.steps)
    value = replica_throughput(angle_pol, dev_s)
    clocks = clk.summary()
    # the same bodies back to back through the single-body sweep
    stages, kernel_s, kernel_w = {}, {}, {}
    e0.record()
    single = []
    for p in probs:
        r = p.sweep("fp32ir")
        single.append(r)
        for kk, v in r.timings.items():
            stages[kk] = stages.get(kk, 0.0) + v
        for kk, v in r.kernel_s.items():
            kernel_s.setdefault(kk, []).extend(v)
            kernel_w.setdefault(kk, []).extend([kernel_work(p, kk)] * len(v))
    e1.record()
    torch.cuda.synchronize()
    b2b_s = e0.elapsed_time(e1) / 1e3
    # FP64 plain on every 16th body; the speed-up is taken on the same bodies
    sample = list(range(0, len(probs), 16))
    t32 = sum(single[i].timings["gpu_total_s"] for i in sample)
    e0.record()
    r64 = {i: probs[i].sweep("fp64") for i in sample}
    e1.record()
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1) / 1e3
    db, rel = 0.0, 0.0
    for i in sample:
        F32, F64 = last[i].dF.sum(0), r64[i].dF.sum(0)
        db = max(db, float(np.max(np.abs(20 * np.log10(np.abs(F32) / np.abs(F64))))))
        rel = max(rel, float(np.max(np.abs(F32 - F64)) / np.max(np.abs(F64))))
    # end to end through the public batch API with host inputs
    t0 = time.perf_counter()
    bs.solve_bor_batch(bodies, thetas, mode_tol=0.0, table_precision="auto")
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    h2d = sum(p.h2d_bytes() for p in probs)
    d2h = sum((p.m_max + 1) * 2 * len(thetas) * 16 + (p.m_max + 1) * 20 for p in probs)
    return dict(adjoint=None, value=value, dev_s=dev_s, stages=stages, kernel_s=kernel_s, kernel_work=kernel_w,
                steps=1, clocks=clocks, launches=launches, f64_s=t64 * dev_s / max(t32, 1e-12),
                f64_steps=1, f64_note=f"FP64 plain on bodies {sample}: {t64:.2f} s vs FP32+IR {t32:.2f} s "
                                      "(single-body sweeps), scaled to the batch by that ratio",
                db=db, rel=rel, e2e_s=e2e_s, h2d=h2d, d2h=d2h,
                refine_iters=max(r.refine_iters for r in last), residual=float(max(np.max(r.residual) for r in last)),
                angle_pol=angle_pol / world * world, M=max(p.m_max for p in probs), thetas=thetas,
                batch={"classes": batch.summary(), "resident": batch.resident(),
                       "back_to_back_s": b2b_s, "back_to_back_angle_pol_s": angle_pol / b2b_s,
                       "batched_s": dev_s, "roofline_note": "roofline and stage times of the back-to-back pass"})


def roofline(res, peaks, workload):
    """Roofline of the kernel with the largest device time per step.

    Launch durations come from CUDA events recorded on the launch stream
    around single launches inside the timed steps; achieved = algorithmic work
    of those launches / their time.  The residual R = B - (Z_far + Z_near) X is
    GEMM-shaped and runs on the tensor cores (13 exact bf16 slice-pair
    products; only the 8 n^2 nrhs useful flops are counted); the fills are arithmetic-bound on the
    CUDA cores and are reported with the flops of their transforms against the
    same compute roof, with the pipe that actually bounds them in a note.
    """
    ks, kw = res["kernel_s"], res["kernel_work"]
    per_step = {k: sum(v) / res["steps"] for k, v in ks.items()}
    name = max(per_step, key=per_step.get)
    t_sum, w_sum = sum(ks[name]), sum(kw[name])
    shares = {k: round(v / res["dev_s"], 4) for k, v in per_step.items()}
    if name.startswith("residual"):
        ach = w_sum / t_sum / 1e12
        peak = peaks["bf16_tflops"]
        out = {"bound": "tensor", "achieved": round(ach, 3), "peak": peak, "unit": "TFLOP/s",
               "frac": round(ach / peak, 5) if peak else None,
               "note": "residual B - Z X of all modes, 8 n^2 nrhs (M+1) useful flops per launch, "
                       "computed as 13 exact bf16 slice-pair products on the tensor cores"}
    else:
        # the fills are compute-bound on the CUDA cores (FP32 pipe and instruction
        # issue); the schema's compute roof is the measured tensor peak, so the
        # FP32-pipe roof (nominal: 152 SMs x 128 FMA lanes x 2 flops x SM clock)
        # and the ncu pipe counters of the committed profile are added
        ach = w_sum / t_sum / 1e12
        peak = peaks["bf16_tflops"]
        fp32_peak = 152 * 128 * 2 * (peaks.get("sm_max_mhz") or 2070.0) * 1e6 / 1e12
        out = {"bound": "tensor", "achieved": round(ach, 3), "peak": peak, "unit": "TFLOP/s",
               "frac": round(ach / peak, 5) if peak else None}
        ctx = FILL_COUNTERS.get(name, {})
        out["fp32_pipe"] = dict({"achieved_tflops": round(ach, 3), "nominal_peak_tflops": round(fp32_peak, 1),
                                 "frac": round(ach / fp32_peak, 4)}, **ctx)
        prob = res.get("prob")
        if name == "far_fill" and prob is not None:
            # the fill's natural unit: Green's-function samples per second
            # (every far Gauss-point pair at every half-grid azimuth node)
            samples = float(4 * prob.N) ** 2 * (prob.n_xi // 2 + 1)
            out["fp32_pipe"]["samples_per_s"] = float(f"{samples * len(ks[name]) / t_sum:.4g}")
        if name == "near_fill":
            out["note"] = ("near fill (CUDA cores, FP32 pipe; no tensor-core work -- the schema's compute roof "
                           "is the bf16 one, fp32_pipe holds the pipe that bounds it): 4 flops per azimuth node "
                           "and order of the cos(m xi) projection; each is a double-float multiply-add on the "
                           "FP32 pipe (~20 FP32 instructions with the recurrence), and every node's "
                           "transcendentals run in double-float as well")
        else:
            out["note"] = ("far fill: 4 flops per far Gauss-point pair, sample and order of the DCT (all "
                           "P^2 pairs; the kernel samples each symmetric pair once and runs the DCT as "
                           "bf16 digit products on the tensor cores); the sampling (double-float phase, "
                           "table-driven sin/cos) and the double-float contraction are not counted")
    out.update({"kernel": name, "launch_ms": round(t_sum / len(ks[name]) * 1e3, 3),
                "launches_per_step": len(ks[name]) / res["steps"], "share_of_step": shares,
                "traffic": TRAFFIC.get((name, workload)), "peak_source": peaks["source"]})
    return out


# DRAM bytes (read + write) per launch of the fills, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum, one pass) of the named workload;
# None where not captured.
TRAFFIC = {     # (kernel, workload) -> bytes per launch
    ("near_fill", "cone_sphere_ka40"): 21.18e6 + 0.07e6,   # inputs only: nodes stay on chip
    ("far_fill", "cone_sphere_ka40"): 13.87e9 + 13.06e9,   # Z_far by FP64 atomics (4.7 GB once)
}

# ncu pipe counters of the fills on the 600-segment cone-sphere (ka = 20), the
# profiles under profiles/ (the same kernels as the bench runs)
FILL_COUNTERS = {
    "far_fill": {"fma_pipe_busy_pct_ncu": 50.9, "issue_active_pct_ncu": 46.5, "tensor_pipe_pct_ncu": 5.95,
                 "profile": "profiles/far_efie_tc_cone_sphere_ka20.md"},
    "near_fill": {"fma_pipe_busy_pct_ncu": 54.4, "issue_active_pct_ncu": 51.7,
                  "profile": "profiles/near_efie_group_cone_sphere_ka20.md"},
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cone_sphere_ka40", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    w = WORKLOADS[args.workload]
    n_theta = int(round((w.get("theta1", 180.0) - w.get("theta0", 0.0)) / w["dtheta"])) + 1
    config = {"workload": args.workload, "body": w["body"], "N": w["N"], "k": w["k"], "m_max": w["M"],
              "n_theta": n_theta, "pols": 2,
              **({"n_bodies": w["n_bodies"], "seed": 0, "N": "200..1600", "k": "12 seg/wavelength",
                  "m_max": "ceil(k rho_max) + 10", "cpu_baseline_sample": "first body"}
                 if w["body"] == "random" else {}),
              "l2": "per-step working set of several GB (>> 129 MB L2)",
              "parallelism": f"replicas x{world}"}
    cores = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        vals, timed, full = [], [], []
        sample = ""
        t_steps = 0.0
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            v, sample, _, sampled, total = cpu_baseline(args.workload, cores)
            if i >= args.warmup:
                t_steps += time.perf_counter() - t0
                vals.append(v)
                timed.append(sampled)
                full.append(total)
        v = statistics.median(vals)
        # each step runs (and times) a bounded sample of the sweep; value is the
        # whole-sweep throughput that the sample implies (angle.pol over the
        # sample's time scaled by element pairs and mode systems)
        line = {"metric": METRIC, "value": v, "unit": "angle·pol/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_steps / args.steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex128",
                "data": "synthetic (seeded geometry)", "config": config, "impl": "reference",
                "timed_per_step": {"sample_s": statistics.median(timed), "step_wall_s": t_steps / args.steps,
                                   "extrapolated_sweep_s": statistics.median(full),
                                   "extrapolation_factor": statistics.median(full) / statistics.median(timed),
                                   "what": "the oracle port (a NumPy/C restatement of the reference's "
                                           "solve_bor) on a bounded sample of the sweep; the reference itself "
                                           "cannot run on the GPU host"},
                "cpu_baseline": {"value": v, "unit": "angle·pol/s", "cores": cores, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": v, "unit": "angle·pol/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_batch(args, rank, world) if w["body"] == "random" else run_gpu(args, rank, world)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        v, sample, _, sampled, total = cpu_baseline(args.workload, cores)
        cpu = {"value": v, "unit": "angle·pol/s", "cores": cores, "kind": "port", "sample": sample,
               "sample_s": sampled, "extrapolated_sweep_s": total}
    peaks = load_peaks()
    line = {
        "metric": METRIC, "value": res["value"], "unit": "angle·pol/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["dev_s"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex64+fp64-refine",
        "data": "synthetic (pinned tangent cone-sphere geometry)", "config": config,
        "e2e": {"value": res["angle_pol"] * world / res["e2e_s"], "unit": "angle·pol/s",
                "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"]},
        "gpu_launches": res["launches"],
        "clocks": res["clocks"],
        "roofline": roofline(res, peaks, args.workload),
        "cpu_baseline": cpu,
        "fp64_plain": {"value": res["angle_pol"] / res["f64_s"], "ms_per_step": res["f64_s"] * 1e3,
                       "steps": res["f64_steps"], **({"note": res["f64_note"]} if "f64_note" in res else {})},
        "speedup_fp32ir_vs_fp64": res["f64_s"] / res["dev_s"],
        "accuracy_vs_fp64": {"max_db_err": res["db"], "max_rel_amp_err": res["rel"], **res.get("acc_extra", {})},
        "refine": {"iters": res["refine_iters"], "max_residual": res["residual"]},
        "stages_s": {k: round(v, 5) for k, v in res["stages"].items()},
    }
    if res.get("vs_ref") is not None:
        line["accuracy_vs_reference"] = res["vs_ref"]
    if res.get("batch") is not None:
        line["batch"] = res["batch"]
    if res["adjoint"] is not None:
        line["adjoint"] = res["adjoint"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
