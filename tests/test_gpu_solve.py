"""End-to-end solve_bor on the GPU vs the reference (goldens) and Mie."""
import math

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def db_err(a, b):
    a, b = np.abs(np.asarray(a)) ** 2, np.abs(np.asarray(b)) ** 2
    return float(np.max(np.abs(10 * np.log10(a / b))))


@pytest.mark.parametrize("name", ["sphere_n24", "conesphere_n40", "openshell_n20"])
def test_solve_fp64_matches_reference(pkg, name):
    D = load_golden(name)
    r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], n_modes=int(D["m_max"]),
                                 mode_tol=0.0, table_precision="double")
    assert rel(r["amp_vv"], D["efie_amp_vv"]) < 1e-10
    assert rel(r["amp_hh"], D["efie_amp_hh"]) < 1e-10
    assert r["linear_residual"] < 1e-12
    assert r["modes_used"] == int(D["m_max"])


@pytest.mark.parametrize("name", ["sphere_n24", "conesphere_n40", "openshell_n20"])
def test_solve_fp32ir_within_tolerance(pkg, name):
    """FP32 fill/LU + FP64 refinement: <= 0.01 dB and 1e-4 relative amplitude."""
    D = load_golden(name)
    r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], n_modes=int(D["m_max"]),
                                 mode_tol=0.0, table_precision="auto")
    assert r["precision"] == "fp32ir"
    for pol in ("vv", "hh"):
        assert rel(r[f"amp_{pol}"], D[f"efie_amp_{pol}"]) < 1e-4
        assert db_err(r[f"amp_{pol}"], D[f"efie_amp_{pol}"]) < 0.01


def test_c1_sphere(pkg):
    """240-segment sphere, ka = 10, |m| <= 20, 181 angles x 2 pols vs the reference and Mie."""
    D = load_golden("c1_sphere")
    for tp, tol in (("double", 1e-10), ("auto", 1e-4)):
        r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], n_modes=20,
                                     mode_tol=0.0, table_precision=tp)
        assert rel(r["amp_vv"], D["amp_vv"]) < tol
        assert rel(r["amp_hh"], D["amp_hh"]) < tol
        assert db_err(r["amp_vv"], D["amp_vv"]) < 0.01
        mie = float(D["mie"])
        assert abs(10 * math.log10(r["sigma_vv"][0] / mie)) < 0.01


def test_mode_truncation_matches_reference_rule(pkg, oracle):
    """mode_tol truncation (two quiet modes) gives the oracle's modes_used and sum."""
    D = load_golden("sphere_n24")
    kw = dict(n_modes=14, mode_tol=1e-6)
    ref = oracle.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], **kw)
    r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], table_precision="double", **kw)
    assert ref["modes_used"] < 14
    assert r["modes_used"] == ref["modes_used"]
    assert rel(r["amp_vv"], ref["amp_vv"]) < 1e-10
