"""Generate the full-size golden fixtures in tests/golden/ by running the
REFERENCE at the benchmark sizes.

Run where the reference tree is mounted; its location comes from the
environment only:

    GHOST_REFERENCE_DIR=<reference tree> python oracle/build_oracle.py
    GHOST_REFERENCE_DIR=<reference tree> python tests/golden/make_fullsize_golden.py c2
    GHOST_REFERENCE_DIR=<reference tree> python tests/golden/make_fullsize_golden.py c5modes
    GHOST_REFERENCE_DIR=<reference tree> python tests/golden/make_fullsize_golden.py bspline_fd

The reference streams its far blocks through its own C sampler
(bor_stream_kernel.c), compiled from the reference's source by
oracle/build_oracle.py into oracle/_ref/; the reference's NumPy fallback gives
bit-equivalent blocks, only slower (bor_streaming.py:80-102).

* ``c2``: the tangent cone-sphere of the precision benchmark (hemisphere
  a = 0.5 m, 15 deg cone, N = 1200 equal-arc segments, k = 80 rad/m, |m| <= 50,
  361 angles 0..180 deg in 0.5 deg steps, VV and HH), solved by the reference's
  solve_bor (EFIE, table_precision="double", assembly="streaming",
  mode_tol=0).  Stored: the 722 complex amplitudes, the linear residual, the
  wall time and the core count of the run.
* ``c5modes``: the same body at N = 3000, k = 200, |m| <= 120 (the large
  benchmark).  A full reference sweep takes many hours, so the fixture holds
  the reference's per-mode far-field contributions dF_|m| (the +m and -m
  systems summed, exactly what the reference's mode loop adds to F,
  bor_solver.py:744-769) for |m| in {0, 60, 120} at 181 angles (1 deg steps),
  from BorPecSolver.enable_streaming / prepare_operators / assemble_mode /
  basis_mask / rhs_mode / np.linalg.solve / farfield_mode.
* ``bspline_fd``: central differences of the reference's FP64 solve_bor for the
  shape-gradient check: the clamped cubic B-spline body with 12 seeded control
  radii U(0.3, 0.6) (seed 0), N = 120, k = 10, |m| <= 12, J = mean of
  sigma_HH (linear m^2) over theta = 30..60 deg in 2.5 deg steps.  Every radius
  is moved by +-1e-4 and +-5e-5 m.
"""

import ctypes
import importlib
import math
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("GHOST_REFERENCE_DIR")
if not REF:
    raise SystemExit("set GHOST_REFERENCE_DIR to the reference tree")
sys.path.insert(0, REF)
sys.path.insert(0, REPO)

import bor_kernels as rk      # noqa: E402  (reference)
import bor_solver as rs       # noqa: E402  (reference)
import bor_streaming as rst   # noqa: E402  (reference)

bodies = importlib.import_module("20260722_ghost_gb300.bodies")
C0 = rk.C0
WORKERS = int(os.environ.get("GHOST_REF_WORKERS", str(os.cpu_count() or 1)))


def _use_reference_sampler():
    """Bind the reference's compiled sampler the way its own loader does
    (bor_streaming.py:50-73), from oracle/_ref/."""
    path = os.path.join(REPO, "oracle", "_ref", "bor_stream_kernel.so")
    if not os.path.exists(path):
        raise SystemExit("build oracle/_ref first: python oracle/build_oracle.py")
    lib = ctypes.CDLL(path)
    dp = ctypes.POINTER(ctypes.c_double)
    ci, cd = ctypes.c_int, ctypes.c_double
    lib.sample_g.argtypes = [ci, ci, ci, dp, dp, dp, dp, cd, dp, dp]
    lib.sample_g.restype = None
    bracket_args = [ci, ci, ci] + [dp] * 8 + [cd, dp, dp] + [dp] * 4
    lib.sample_mfie.argtypes = bracket_args
    lib.sample_mfie.restype = None
    lib.sample_ibc.argtypes = bracket_args
    lib.sample_ibc.restype = None
    rst._NATIVE = lib


def _host():
    return {"host_cores": os.cpu_count() or 1, "workers": WORKERS,
            "host_machine": platform.machine(), "host_cpu": platform.processor() or ""}


def c2():
    pts = bodies.cone_sphere_generatrix(0.5, 15.0, 1200)
    k = 80.0
    f = k * C0 / (2.0 * math.pi)
    th = np.arange(0.0, 180.0 + 1e-9, 0.5)
    t = time.time()
    r = rs.solve_bor(pts, f, th, formulation="efie", n_modes=50, mode_tol=0.0,
                     workers=WORKERS, table_precision="double", assembly="streaming")
    wall = time.time() - t
    print(f"C2 reference solve_bor: {wall:.1f} s on {WORKERS} workers, "
          f"residual {r['linear_residual']:.2e}", flush=True)
    np.savez_compressed(os.path.join(HERE, "c2_conesphere_ref.npz"),
                        points=pts, freq_hz=f, k=k, m_max=50, thetas=th,
                        amp_vv=np.array(r["amp_vv"]), amp_hh=np.array(r["amp_hh"]),
                        residual=r["linear_residual"], wall_s=wall,
                        modes_used=r["modes_used"], **_host())


def c5modes(modes=(0, 60, 120)):
    n, k, M = 3000, 200.0, 120
    pts = bodies.cone_sphere_generatrix(0.5, 15.0, n)
    f = k * C0 / (2.0 * math.pi)
    th = np.arange(0.0, 180.0 + 1e-9, 1.0)
    t0 = time.time()
    s = rs.BorPecSolver(pts, f)
    # mode blocks of WORKERS modes: a block holds 9 order primitives of
    # (block + 2) orders at Nn^2 complex128 each
    s.enable_streaming(M, efie=True, mfie=False, single_blocks=False,
                       workers=WORKERS, mode_block=WORKERS)
    s.prepare_operators(M, efie=True, mfie=False, ibc=False, workers=WORKERS)
    t_prep = time.time() - t0
    print(f"C5 prepare: {t_prep:.1f} s", flush=True)
    out = {"points": pts, "freq_hz": f, "k": k, "m_max": M, "thetas": th,
           "modes": np.asarray(modes, int), **_host()}
    n_dofs = 2 * s.Nn
    for am in modes:
        t = time.time()
        dF = np.zeros((2, len(th)), np.complex128)
        res = 0.0
        for m in ([0] if am == 0 else [am, -am]):
            Z = s.assemble_mode(m, M)
            mask = s.basis_mask(m)
            A = Z[np.ix_(mask, mask)]
            B = np.stack([s.rhs_mode(m, tt, pol)[mask] for tt in th for pol in ("VV", "HH")],
                         axis=1)
            X = np.linalg.solve(A, B)
            res = max(res, float(np.linalg.norm(A @ X - B) / np.linalg.norm(B)))
            ci = 0
            for it, tt in enumerate(th):
                for ip, pol in enumerate(("VV", "HH")):
                    sol = np.zeros(n_dofs, np.complex128)
                    sol[mask] = X[:, ci]
                    ci += 1
                    fth, fph = s.farfield_mode(m, sol, tt)
                    dF[ip, it] += fth if pol == "VV" else fph
        out[f"dF_{am}"] = dF
        out[f"residual_{am}"] = res
        out[f"wall_{am}"] = time.time() - t
        print(f"C5 |m| = {am}: {time.time() - t:.1f} s, residual {res:.2e}", flush=True)
        np.savez_compressed(os.path.join(HERE, "c5_conesphere_modes_ref.npz"), **out)
    print(f"C5 modes total {time.time() - t0:.1f} s", flush=True)


def bspline_fd():
    radii = np.random.default_rng(0).uniform(0.3, 0.6, 12)
    n_seg, k, M = 120, 10.0, 12
    f = k * C0 / (2.0 * math.pi)
    th = np.arange(30.0, 60.0 + 1e-9, 2.5)

    def J(r):
        pts, _ = bodies.bspline_body(r, n_seg)
        res = rs.solve_bor(pts, f, th, formulation="efie", n_modes=M, mode_tol=0.0,
                           workers=WORKERS, table_precision="double", assembly="streaming")
        return float(np.mean(res["sigma_hh"]))

    t = time.time()
    out = {"radii": radii, "n_seg": n_seg, "k": k, "freq_hz": f, "m_max": M,
           "thetas": th, "J0": J(radii)}
    for h, tag in ((1e-4, "h1"), (5e-5, "h2")):
        jp = np.empty(len(radii))
        jm = np.empty(len(radii))
        for j in range(len(radii)):
            rp, rm = radii.copy(), radii.copy()
            rp[j] += h
            rm[j] -= h
            jp[j], jm[j] = J(rp), J(rm)
        out[f"{tag}"] = h
        out[f"Jp_{tag}"] = jp
        out[f"Jm_{tag}"] = jm
        print(f"bspline FD h = {h}: {time.time() - t:.1f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, "bspline_fd_ref.npz"), **out)


if __name__ == "__main__":
    _use_reference_sampler()
    what = sys.argv[1:] or ["c2"]
    for w in what:
        {"c2": c2, "c5modes": c5modes, "bspline_fd": bspline_fd}[w]()
