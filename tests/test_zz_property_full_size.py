"""Size-independent properties at the full C2 size (GPU).

At axial incidence (theta = 0 and 180 degrees) the two polarisations of a body
of revolution are a 90-degree rotation about its axis apart, so the monostatic
amplitudes agree: F_VV = F_HH (checked to 1e-15 on the oracle, EFIE and
CFIE).  Here the FP32+IR sweep of the full 1200-segment cone-sphere at ka = 40
with |m| <= 50 must keep that to 1e-6 of its largest amplitude.  Named to run after
the parity tests, so a failure here does not hide their results.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("formulation", ["efie", "cfie"])
def test_axial_incidence_polarisations_agree_at_c2_size(pkg, formulation):
    pts = pkg.bodies.cone_sphere_generatrix(0.5, 15.0, 1200)
    f = 80.0 * 299792458.0 / (2 * math.pi)
    r = pkg.bor_solver.solve_bor(pts, f, [0.0, 90.0, 180.0], formulation=formulation, n_modes=50,
                                 mode_tol=0.0, table_precision="auto")
    vv, hh = np.array(r["amp_vv"]), np.array(r["amp_hh"])
    peak = float(np.max(np.abs(np.r_[vv, hh])))
    for i in (0, 2):
        assert abs(vv[i] - hh[i]) <= 1e-6 * peak, (i, abs(vv[i] - hh[i]) / peak)
    assert r["linear_residual"] < 1e-6
