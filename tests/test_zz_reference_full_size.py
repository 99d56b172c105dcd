"""Full-size parity with the reference: the 1200-segment tangent cone-sphere of
the precision benchmark (a = 0.5 m, 15 deg cone, k = 80, |m| <= 50, 361 angles,
VV and HH), against the amplitudes of the reference's own FP64 solve_bor
(EFIE, table_precision="double", assembly="streaming", mode_tol=0) stored in
tests/golden/c2_conesphere_ref.npz by tests/golden/make_fullsize_golden.py.

The plain FP64 GPU path must agree to 1e-10 of the largest amplitude; the
FP32 + FP64-refinement path (tensor-core far fill, exact residual updates) to
1e-4 relative and 0.01 dB at every angle and polarisation.

The large benchmark body (N = 3000, k = 200, |m| <= 120) is checked mode by
mode: tests/golden/c5_conesphere_modes_ref.npz holds the reference's FP64
per-|m| far-field contributions (the +m and -m systems summed, as its mode
loop adds them) for |m| in {0, 60, 120} at 181 angles, and the FP32 +
refinement sweep's contributions of those modes must agree with them.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    return load_golden("c2_conesphere_ref")


def _errors(r, D):
    out = {}
    for pol in ("vv", "hh"):
        a = np.asarray(r[f"amp_{pol}"])
        b = D[f"amp_{pol}"]
        out[pol] = (float(np.max(np.abs(a - b)) / np.max(np.abs(b))),
                    float(np.max(np.abs(20 * np.log10(np.abs(a) / np.abs(b))))))
    return out


@pytest.mark.parametrize("precision,rel_tol,db_tol", [("double", 1e-10, 1e-4), ("auto", 1e-4, 0.01)])
def test_c2_cone_sphere_matches_reference(pkg, ref, precision, rel_tol, db_tol):
    r = pkg.bor_solver.solve_bor(ref["points"], float(ref["freq_hz"]), ref["thetas"], n_modes=int(ref["m_max"]),
                                 mode_tol=0.0, table_precision=precision)
    err = _errors(r, ref)
    print(f"\n{precision}: {err}")
    for pol, (rel, db) in err.items():
        assert rel < rel_tol, (pol, rel)
        assert db < db_tol, (pol, db)


def test_c5_cone_sphere_modes_match_reference(pkg):
    D = load_golden("c5_conesphere_modes_ref")
    modes = [int(m) for m in D["modes"] if f"dF_{int(m)}" in D]
    assert modes
    prob = pkg.engine.BorGpuProblem(D["points"], float(D["freq_hz"]), D["thetas"], m_max=int(D["m_max"]))
    r = prob.sweep("fp32ir")
    top = max(float(np.max(np.abs(D[f"dF_{m}"]))) for m in modes)
    for m in modes:
        ref_m = D[f"dF_{m}"]
        err = float(np.max(np.abs(r.dF[m] - ref_m)))
        own = float(np.max(np.abs(ref_m)))
        print(f"\n|m| = {m}: max |dF| {own:.3e}, error {err / own:.3e} of the mode, {err / top:.3e} of the largest")
        assert err < 1e-6 * own + 1e-9 * top, (m, err / own)
