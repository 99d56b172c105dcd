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
}
METRIC = "monostatic RCS angle·pol/s on 1 GB300: FP32+IR batched vs FP64 plain, ≤0.01 dB err"


def workload_inputs(name):
    import numpy as np
    w = WORKLOADS[name]
    bodies = importlib.import_module(PKG + ".bodies")
    if w["body"] == "sphere":
        pts = bodies.sphere_generatrix(w["a"], w["N"])
    else:
        pts = bodies.cone_sphere_generatrix(w["a"], w["half_angle"], w["N"])
    thetas = np.arange(0.0, 180.0 + 1e-9, w["dtheta"])
    return pts, w["k"] * C0 / (2 * math.pi), thetas, w["M"]


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
        return {"hbm_gbs": d.get("hbm_gbs"), "bf16_tflops": d.get("bf16_tflops"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port of the reference algorithm on the host cores
# ---------------------------------------------------------------------------

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
    # one |m|: complete near cache is needed by assemble; fill the rest untimed
    s.prepare(M, efie=True, workers=cores, pairs=[p for p in pairs if p not in set(sub)])
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
    sample = (f"oracle port of the reference sweep on {cores} host threads: far sweep over "
              f"{n_far}/{ne} test elements, {len(sub)}/{len(pairs)} near element pairs, one |m| "
              f"(m=+-{am}) solved for all {2 * len(thetas)} columns; extrapolated to {2 * M + 1} "
              f"mode systems ({total:.0f} s per sweep)")
    return 2 * len(thetas) / total, sample, time.perf_counter() - t_start


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
        kernel_s = {}
        for _ in range(args.steps):
            r = prob.sweep("fp32ir")
            results.append(r)
            for kk, v in r.timings.items():
                stages[kk] = stages.get(kk, 0.0) + v / args.steps
            for kk, v in r.kernel_s.items():
                kernel_s.setdefault(kk, []).extend(v)
        e1.record()
        torch.cuda.synchronize()
        barrier()
    launches = nat.launch_count() - l0
    dev_s = e0.elapsed_time(e1) / 1e3 / args.steps
    if dist:
        t = torch.tensor([dev_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_s = float(t)
    value = angle_pol * world / dev_s
    clocks = clk.summary()

    # FP64 plain comparator (same sweep, FP64 fill/LU/solve/residual)
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
    db = float(np.max(np.abs(20 * np.log10(np.abs(F32) / np.abs(F64)))))
    rel = float(np.max(np.abs(F32 - F64)) / np.max(np.abs(F64)))

    # end to end through the public API with host inputs
    bs.solve_bor(pts, f, thetas, n_modes=M, mode_tol=0.0, table_precision="auto")
    torch.cuda.synchronize()
    barrier()
    e2e_steps = max(1, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        out = bs.solve_bor(pts, f, thetas, n_modes=M, mode_tol=0.0, table_precision="auto")
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t)
    h2d = prob.h2d_bytes()
    d2h = (M + 1) * angle_pol * 16 + (M + 1) * (2 * 8 + 4)
    return dict(value=value, dev_s=dev_s, stages=stages, kernel_s=kernel_s, clocks=clocks, launches=launches,
                f64_s=f64_s, f64_steps=f64_steps, db=db, rel=rel, e2e_s=e2e_s, h2d=h2d, d2h=d2h,
                refine_iters=results[-1].refine_iters, residual=float(np.max(results[-1].residual)),
                prob=prob, angle_pol=angle_pol, M=M, thetas=thetas)


def roofline(res, peaks):
    """Roofline of the kernel with the largest device time per step.

    Launch durations come from CUDA events recorded on the launch stream
    around single launches inside the timed steps.  Algorithmic work per
    launch:
      residual  R = B - (Z_far + Z_near) X over every mode: 8 n^2 nrhs (M+1)
                real flops (complex MAC = 8); a GEMM, so the tensor peak is
                the ceiling even though the kernel runs split-word FP32 on
                the CUDA cores
      fills     far_fill / near_fill: the bytes of the operator they write
                (complex128 Z(m) for m = 0..M, resp. the near band); both
                are arithmetic-bound, so this fraction is small by nature
    """
    prob = res["prob"]
    ks = res["kernel_s"]
    steps = max(1, len(ks.get("far_fill", [1])))
    per_step = {k: sum(v) / steps for k, v in ks.items()}
    name = max(per_step, key=per_step.get)
    dur = statistics.mean(ks[name])
    n, M1, nrhs = prob.n, prob.m_max + 1, prob.nrhs
    shares = {k: round(v / res["dev_s"], 4) for k, v in per_step.items()}
    if name == "residual":
        work = 8.0 * n * n * nrhs * M1
        ach = work / dur / 1e12
        peak = peaks["bf16_tflops"]
        out = {"bound": "tensor", "achieved": round(ach, 3), "peak": peak, "unit": "TFLOP/s",
               "frac": round(ach / peak, 5) if peak else None,
               "note": "residual B - Z X of all modes, 8 n^2 nrhs (M+1) flops per launch; "
                       "split-word FP32 on CUDA cores, so the bf16 tensor peak is a loose ceiling"}
    else:
        work = 16.0 * M1 * (n * n if name == "far_fill" else 4 * prob.Nn * 5)
        ach = work / dur / 1e9
        peak = peaks["hbm_gbs"]
        out = {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
               "frac": round(ach / peak, 4) if peak else None,
               "note": f"{name}: complex128 operator bytes written per launch"}
    out.update({"kernel": name, "launch_ms": round(dur * 1e3, 3), "launches_per_step":
                len(ks[name]) / steps, "share_of_step": shares, "traffic": TRAFFIC.get(name),
                "peak_source": peaks["source"]})
    return out


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the 1200-segment
# cone-sphere; None until captured.
TRAFFIC = {}


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
    config = {"workload": args.workload, "body": w["body"], "N": w["N"], "k": w["k"], "m_max": w["M"],
              "n_theta": int(round(180 / w["dtheta"])) + 1, "pols": 2,
              "l2": "per-step working set of several GB (>> 129 MB L2)",
              "parallelism": f"replicas x{world}"}
    cores = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        vals = []
        sample = ""
        for i in range(args.warmup + args.steps):
            v, sample, _ = cpu_baseline(args.workload, cores)
            if i >= args.warmup:
                vals.append(v)
        v = statistics.median(vals)
        line = {"metric": METRIC, "value": v, "unit": "angle·pol/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 2 * config["n_theta"] / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "complex128",
                "data": "synthetic (seeded geometry)", "config": config, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": "angle·pol/s", "cores": cores, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": v, "unit": "angle·pol/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_gpu(args, rank, world)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        v, sample, _ = cpu_baseline(args.workload, cores)
        cpu = {"value": v, "unit": "angle·pol/s", "cores": cores, "kind": "port", "sample": sample}
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
        "roofline": roofline(res, peaks),
        "cpu_baseline": cpu,
        "fp64_plain": {"value": res["angle_pol"] / res["f64_s"], "ms_per_step": res["f64_s"] * 1e3,
                       "steps": res["f64_steps"]},
        "speedup_fp32ir_vs_fp64": res["f64_s"] / res["dev_s"],
        "accuracy_vs_fp64": {"max_db_err": res["db"], "max_rel_amp_err": res["rel"]},
        "refine": {"iters": res["refine_iters"], "max_residual": res["residual"]},
        "stages_s": {k: round(v, 5) for k, v in res["stages"].items()},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
