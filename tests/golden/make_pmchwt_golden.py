"""Generate tests/golden/pmchwt_sphere_n24.npz, coated_sphere.npz and
layered_sphere.npz by running the REFERENCE's PMCHWT paths
(bor_solver.solve_bor_dielectric, BorCrossOperators, solve_bor_coated_pec,
solve_bor_coated2_pec).

Run where the reference tree is mounted (its location from GHOST_REFERENCE_DIR):

    python tests/golden/make_pmchwt_golden.py        # ~1 min

Stored (FP64): a 24-segment sphere (a = 0.5 m, ka = 2); for a lossy
dielectric medium the interior EFIE operator T_i and the PMCHWT operators P_e
(air) and P_i of modes 0 and 2; full solves for a lossy, a lossless and a
lossy magnetic medium; the dielectric-sphere Mie backscatter of a few cases.
Coated: a 12-segment PEC sphere (0.4 m) inside a 16-segment coating (0.5 m),
ka = 1.5; the cross operators T and P between the two surfaces (both
directions) for mode 1; a full solve; the coated-sphere Mie backscatter.
Layered: a PEC sphere under two full layers (three closed surfaces), one solve.
"""

import importlib
import math
import os
import sys

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

MEDIA = [(2.5 - 0.2j, 1.0), (4.0, 1.0), (2.0 - 0.1j, 1.5 - 0.2j)]


def main():
    pts = bodies.sphere_generatrix(0.5, 24)
    k = 4.0
    f = k * rk.C0 / (2.0 * math.pi)
    m_max = 8
    thetas = np.arange(0.0, 180.0001, 30.0)
    out = {"points": pts, "freq_hz": f, "k": k, "m_max": m_max, "thetas": thetas,
           "media": np.array(MEDIA, dtype=complex), "modes": np.array([0, 2])}
    se = rs.BorPecSolver(pts, f)
    si = rs.BorPecSolver(pts, f, medium=MEDIA[0])
    for s in (se, si):
        s.prepare_operators(m_max, efie=True, ibc=True, workers=8)
    for m in out["modes"]:
        out[f"Ti_{m}"] = si.assemble_mode(int(m), m_max)
        out[f"Pe_{m}"] = se.assemble_pmchwt_P(int(m), m_max)
        out[f"Pi_{m}"] = si.assemble_pmchwt_P(int(m), m_max)
    for i, (eps, mu) in enumerate(MEDIA):
        r = rs.solve_bor_dielectric(pts, f, thetas, eps, mu, n_modes=m_max, mode_tol=0.0, workers=8)
        out[f"amp_vv_{i}"] = np.array(r["amp_vv"])
        out[f"amp_hh_{i}"] = np.array(r["amp_hh"])
    cases = [(0.5, 300e6, 2.5, 1.0), (0.3, 1e9, 4.0 - 0.5j, 1.0), (1.0, 200e6, 2.0 - 0.1j, 1.5 - 0.2j),
             (0.2, 2e9, 10.0, 1.0)]
    out["mie_cases"] = np.array([[a, fr, complex(e).real, complex(e).imag, complex(u).real, complex(u).imag]
                                 for a, fr, e, u in cases])
    out["mie_sigma"] = np.array([rmie.sigma_dielectric_sphere(a, e, u, fr) for a, fr, e, u in cases])
    np.savez_compressed(os.path.join(HERE, "pmchwt_sphere_n24.npz"), **out)
    coated()
    print("written")


def coated():
    outer, core = bodies.sphere_generatrix(0.5, 16), bodies.sphere_generatrix(0.4, 12)
    k, m_max, eps, mu = 3.0, 4, 2.5 - 0.3j, 1.0
    f = k * rk.C0 / (2.0 * math.pi)
    thetas = np.arange(0.0, 180.0001, 45.0)
    out = {"outer": outer, "core": core, "freq_hz": f, "m_max": m_max, "thetas": thetas,
           "eps": eps, "mu": mu}
    sLo = rs.BorPecSolver(outer, f, medium=(eps, mu))
    sLc = rs.BorPecSolver(core, f, medium=(eps, mu))
    Xoc, Xco = rs.BorCrossOperators(sLo, sLc), rs.BorCrossOperators(sLc, sLo)
    for X, tag in ((Xoc, "oc"), (Xco, "co")):
        X.prepare(m_max)
        out[f"T_{tag}"] = X.assemble_T(1, m_max)
        out[f"P_{tag}"] = X.assemble_P(1, m_max)
    r = rs.solve_bor_coated_pec(outer, core, f, thetas, eps, mu, n_modes=m_max, mode_tol=0.0, workers=8)
    out["amp_vv"], out["amp_hh"] = np.array(r["amp_vv"]), np.array(r["amp_hh"])
    cases = [(0.4, 0.5, 300e6, 2.5 - 0.3j, 1.0), (0.2, 0.3, 1e9, 4.0, 1.0),
             (0.8, 1.0, 200e6, 2.0 - 0.1j, 1.5 - 0.2j)]
    out["mie_cases"] = np.array([[b, a, fr, complex(e).real, complex(e).imag, complex(u).real,
                                  complex(u).imag] for b, a, fr, e, u in cases])
    out["mie_sigma"] = np.array([rmie.sigma_coated_pec_sphere(b, a, e, u, fr) for b, a, fr, e, u in cases])
    np.savez_compressed(os.path.join(HERE, "coated_sphere.npz"), **out)
    layered()


def layered():
    """Two full layers over a PEC core (the multi-region system without junctions)."""
    outer, mid, core = (bodies.sphere_generatrix(0.5, 14), bodies.sphere_generatrix(0.42, 12),
                        bodies.sphere_generatrix(0.35, 10))
    f = 3.0 * rk.C0 / (2.0 * math.pi)
    thetas = np.arange(0.0, 180.0001, 60.0)
    media = (2.0 - 0.1j, 1.0, 3.0 - 0.4j, 1.2)          # inner eps, mu; outer eps, mu
    r = rs.solve_bor_coated2_pec(outer, mid, core, f, thetas, *media, n_modes=3, mode_tol=0.0,
                                 workers=8)
    np.savez_compressed(os.path.join(HERE, "layered_sphere.npz"), outer=outer, mid=mid, core=core,
                        freq_hz=f, thetas=thetas, media=np.array(media, dtype=complex), m_max=3,
                        amp_vv=np.array(r["amp_vv"]), amp_hh=np.array(r["amp_hh"]),
                        n_unknowns=r["n_unknowns"])


if __name__ == "__main__":
    main()
