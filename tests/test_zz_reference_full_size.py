"""Full-size parity with the reference: the 1200-segment tangent cone-sphere of
the precision benchmark (a = 0.5 m, 15 deg cone, k = 80, |m| <= 50, 361 angles,
VV and HH), against the amplitudes of the reference's own FP64 solve_bor
(EFIE, table_precision="double", assembly="streaming", mode_tol=0) stored in
tests/golden/c2_conesphere_ref.npz by tests/golden/make_fullsize_golden.py.

The plain FP64 GPU path must agree to 1e-10 of the largest amplitude; the
FP32 + FP64-refinement path (tensor-core far fill, exact residual updates) to
1e-4 relative and 0.01 dB at every angle and polarisation.
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
