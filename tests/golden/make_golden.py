"""Generate the golden fixtures in tests/golden/ by running the REFERENCE.

Run in a container where the reference tree is mounted (its location from
GHOST_REFERENCE_DIR):

    python tests/golden/make_golden.py            # small fixtures (~1 min)
    python tests/golden/make_golden.py --c1       # + the 240-segment sphere (~3 min)

Every fixture holds the inputs and the reference's own outputs, FP64, for
the PEC BoR path: per-mode impedance matrices (EFIE and MFIE), excitation
vectors, near/far modal kernels and final complex far-field amplitudes.  The
reference runs with table_precision="double", assembly="streaming" and
mode_tol=0, i.e. exactly the configuration the oracle restates.
"""

import importlib
import math
import os
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
import mie_sphere as rmie     # noqa: E402  (reference)

bodies = importlib.import_module("20260722_ghost_gb300.bodies")
C0 = rk.C0


def freq_for_k(k):
    return k * C0 / (2.0 * math.pi)


def solver_case(name, points, k, m_max, thetas, modes, cfie=True, workers=8):
    """Per-mode operators + full solves of one body."""
    f = freq_for_k(k)
    out = {"points": np.asarray(points, float), "freq_hz": f, "k": k,
           "m_max": m_max, "thetas": np.asarray(thetas, float),
           "modes": np.asarray(modes, int)}
    s = rs.BorPecSolver(points, f)
    s.enable_streaming(m_max, efie=True, mfie=cfie)
    s.prepare_operators(m_max, efie=True, mfie=cfie)
    for m in modes:
        out[f"Ze_{m}"] = s.assemble_mode(m, m_max)
        if cfie:
            out[f"Zm_{m}"] = s.assemble_mfie_mode(m, m_max)
        out[f"mask_{m}"] = s.basis_mask(m)
        for pol in ("VV", "HH"):
            out[f"Ve_{m}_{pol}"] = np.stack([s.rhs_mode(m, th, pol) for th in thetas])
            if cfie:
                out[f"Vm_{m}_{pol}"] = np.stack([s.rhs_mfie_mode(m, th, pol) for th in thetas])
        # far field of a fixed pseudo-random current vector, every angle
        rng = np.random.default_rng(1000 + m)
        x = rng.standard_normal(2 * s.Nn) + 1j * rng.standard_normal(2 * s.Nn)
        out[f"ffx_{m}"] = x
        out[f"ff_{m}"] = np.array([s.farfield_mode(m, x, th) for th in thetas])
    for form in (("efie", "cfie") if cfie else ("efie",)):
        t = time.time()
        r = rs.solve_bor(points, f, thetas, formulation=form, n_modes=m_max,
                         mode_tol=0.0, workers=workers, table_precision="double",
                         assembly="streaming")
        out[f"{form}_amp_vv"] = np.array(r["amp_vv"])
        out[f"{form}_amp_hh"] = np.array(r["amp_hh"])
        out[f"{form}_residual"] = r["linear_residual"]
        print(f"  {name} {form}: {time.time() - t:.1f}s residual {r['linear_residual']:.2e}")
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def kernels_case():
    """Near/far modal kernels and quadrature tables at chosen point pairs."""
    rng = np.random.default_rng(7)
    out = {}
    k, m_max = 9.0, 7
    # near pairs: small separations, some on / touching the axis
    n = 40
    rp = rng.uniform(0.0, 1.0, n); rq = rp + rng.uniform(-0.02, 0.02, n)
    rq = np.abs(rq); rp[:3] = 0.0
    zp = rng.uniform(-1, 1, n); zq = zp + rng.uniform(-0.02, 0.02, n)
    zq[5] = zp[5]; rq[5] = rp[5]          # exact coincidence
    out.update(near_rp=rp, near_zp=zp, near_rq=rq, near_zq=zq, near_k=k, near_m_max=m_max)
    out["near_G"] = rk.modal_kernels_near(rp, zp, rq, zq, k, m_max)
    trp = rng.uniform(-1, 1, n); tzp = np.sqrt(1 - trp ** 2)
    trq = rng.uniform(-1, 1, n); tzq = -np.sqrt(1 - trq ** 2)
    out.update(near_trp=trp, near_tzp=tzp, near_trq=trq, near_tzq=tzq)
    sel = slice(6, n)                     # MFIE brackets need non-coincident pairs
    for name, K in zip(("tt", "tf", "ft", "ff"),
                       rk.mfie_kernels_near(rp[sel], zp[sel], trp[sel], tzp[sel],
                                            rq[sel], zq[sel], trq[sel], tzq[sel], k, m_max)):
        out[f"near_K_{name}"] = K
    # far pairs via the FFT path
    fp = rng.uniform(0.05, 1.0, (2, 30)); fz = rng.uniform(-1, 1, (2, 30))
    out.update(far_rp=fp[0], far_rq=fp[1], far_zp=fz[0], far_zq=fz[1])
    out["far_G"] = rk.modal_kernels_fft(fp[0], fz[0], fp[1], fz[1], k, m_max, n_xi=128)
    for name, K in zip(("tt", "tf", "ft", "ff"),
                       rk.mfie_kernels_fft(fp[0], fz[0], trp[:30], tzp[:30],
                                           fp[1], fz[1], trq[:30], tzq[:30], k, m_max, n_xi=256)):
        out[f"far_K_{name}"] = K
    for kind in ("diag", "corner10", "corner01"):
        s, sp_, w = rs._cell_points(kind)
        out[f"cells_{kind}"] = np.stack([s, sp_, w])
    import bor_streaming as rst
    out["n_xi"] = np.array([[rst._n_xi_efie(kk, r, mm), rst._n_xi_bracket(kk, r, mm)]
                            for kk, r, mm in ((10, 1, 20), (80, .5, 50), (200, .5, 120),
                                              (40, .6, 30), (3, .1, 2))])
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **out)


def mie_case():
    a = 1.0
    kas = np.array([0.1, 0.5, 1.0, 2.0, 5.0, 10.0, 20.0])
    sig = np.array([rmie.sigma_pec_sphere(a, freq_for_k(ka / a)) for ka in kas])
    np.savez_compressed(os.path.join(HERE, "mie.npz"), ka=kas, a=a, sigma=sig)


def main():
    t0 = time.time()
    kernels_case()
    mie_case()
    th = np.arange(0.0, 181.0, 15.0)
    solver_case("sphere_n24", rs.sphere_generatrix(1.0, 24), 2.0, 6, th, [0, 1, -1, 2, 6])
    solver_case("conesphere_n40", bodies.cone_sphere_generatrix(0.5, 15.0, 40), 6.0, 8,
                np.arange(0.0, 181.0, 10.0), [0, 1, 3, -3, 8])
    # open shell: north pole to the equator (one end on the axis, one open end)
    th_open = np.linspace(0.0, 0.5 * math.pi, 21)
    shell = np.column_stack([np.sin(th_open), np.cos(th_open)])
    solver_case("openshell_n20", shell, 2.5, 5, np.arange(0.0, 181.0, 20.0), [0, 1, 2],
                cfie=False)
    if "--c1" in sys.argv:
        f = freq_for_k(10.0)
        pts = rs.sphere_generatrix(1.0, 240)
        th = np.arange(0.0, 181.0, 1.0)
        t = time.time()
        r = rs.solve_bor(pts, f, th, formulation="efie", n_modes=20, mode_tol=0.0,
                         workers=8, table_precision="double", assembly="streaming")
        print(f"  C1 sphere efie: {time.time() - t:.1f}s")
        np.savez_compressed(os.path.join(HERE, "c1_sphere.npz"), points=pts, freq_hz=f,
                            k=10.0, m_max=20, thetas=th,
                            amp_vv=np.array(r["amp_vv"]), amp_hh=np.array(r["amp_hh"]),
                            residual=r["linear_residual"],
                            mie=rmie.sigma_pec_sphere(1.0, f))
    print(f"golden fixtures written in {time.time() - t0:.1f}s")


if __name__ == "__main__":
    main()
