"""Generate tests/golden/ibc_conesphere_n40.npz by running the REFERENCE's
surface-impedance (IBC-EFIE) path.

Run where the reference tree is mounted (its location from GHOST_REFERENCE_DIR):

    python tests/golden/make_ibc_golden.py        # ~1 min

Stored (FP64, the reference with table_precision="double",
assembly="streaming", mode_tol=0): a 40-segment tangent cone-sphere (ka = 6)
with a tapered complex Z_s per element; the per-mode IBC operator additions
``assemble_ibc_extra`` (far streamed brackets + near brackets + Z_s mass
term) for a few modes; full-solve amplitudes with that taper and with a
scalar Z_s; and the impedance-sphere Mie backscatter for a few (ka, Z_s).
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


def main():
    pts = bodies.cone_sphere_generatrix(0.3, 15.0, 40)
    k = 20.0
    f = k * rk.C0 / (2.0 * math.pi)
    ne = len(pts) - 1
    s = (np.arange(ne) + 0.5) / ne
    zs_taper = (60.0 + 240.0 * s) - 1j * (30.0 + 20.0 * np.cos(3.0 * s))
    zs_taper[:5] = 0.0                    # a bare (PEC) nose: source weights vanish there
    m_max = 9
    modes = [0, 1, -4]
    thetas = np.arange(0.0, 180.0001, 15.0)
    out = {"points": pts, "freq_hz": f, "k": k, "m_max": m_max, "modes": np.array(modes),
           "zs_taper": zs_taper, "thetas": thetas}

    zs_pt = None
    solver = rs.BorPecSolver(pts, f)
    zs_pt = zs_taper[solver.g.elem]
    solver.enable_streaming(m_max, efie=True, mfie=False, ibc_zs_pt=zs_pt)
    solver.prepare_operators(m_max, efie=True, mfie=False, ibc=True)
    for m in modes:
        out[f"Zi_{m}"] = solver.assemble_ibc_extra(m, m_max, zs_pt, zs_taper)
    for tag, zs in (("taper", zs_taper), ("scalar", 120.0 - 80.0j)):
        r = rs.solve_bor(pts, f, thetas, formulation="efie", zs=zs, n_modes=m_max, mode_tol=0.0,
                         table_precision="double", assembly="streaming", workers=8)
        out[f"amp_vv_{tag}"] = np.array(r["amp_vv"])
        out[f"amp_hh_{tag}"] = np.array(r["amp_hh"])
    cases = [(1.0, 477.1e6, 0.0), (0.5, 300e6, 50 - 20j), (1.0, 477.1e6, rk.ETA0),
             (0.3, 1e9, 100 + 100j), (2.0, 200e6, 20j)]
    out["mie_cases"] = np.array([[a, fr, complex(z).real, complex(z).imag] for a, fr, z in cases])
    out["mie_sigma"] = np.array([rmie.sigma_impedance_sphere(a, fr, z) for a, fr, z in cases])
    np.savez_compressed(os.path.join(HERE, "ibc_conesphere_n40.npz"), **out)
    print("written; |Zi_0| max", np.max(np.abs(out["Zi_0"])))


if __name__ == "__main__":
    main()
