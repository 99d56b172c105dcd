"""CFIE / MFIE on the GPU: MFIE operator, excitation and full solves against
the reference goldens and the oracle."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

CFIE_CASES = ["sphere_n24", "conesphere_n40"]


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def db_err(a, b):
    a, b = np.abs(np.asarray(a)) ** 2, np.abs(np.asarray(b)) ** 2
    return float(np.max(np.abs(10 * np.log10(a / b))))


@pytest.mark.parametrize("name", CFIE_CASES)
def test_far_bracket_blocks(pkg, oracle, name):
    """Fused MFIE far fill (FP64 and FP32 transforms) vs the oracle's
    streamed bracket blocks, every mode -M..M."""
    D = load_golden(name)
    M = int(D["m_max"])
    o = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    o.build_far(M, efie=False, mfie=True)
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]))
    for dtype, tol in ((np.complex128, 1e-12), (np.complex64, 1e-5)):
        s.enable_streaming(M, efie=False, mfie=True, single_blocks=dtype == np.complex64)
        for m in range(-M, M + 1):
            got = s._stream.bracket_blocks("mfie", m)
            want = [o.Kb[uv, m + M] for uv in range(4)]
            scale = max(np.max(np.abs(w)) for w in want)
            err = max(np.max(np.abs(g - w)) for g, w in zip(got, want)) / scale
            assert err < tol, (dtype, m, err)


@pytest.mark.parametrize("name", CFIE_CASES)
def test_mfie_operator_and_excitation(pkg, name):
    """assemble_mfie_mode (far + near + mass) and rhs_mfie_mode vs the reference goldens."""
    D = load_golden(name)
    M = int(D["m_max"])
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]))
    s.prepare_operators(M, efie=True, mfie=True)
    for m in D["modes"]:
        m = int(m)
        assert rel(s.assemble_mfie_mode(m, M), D[f"Zm_{m}"]) < 1e-12, m
        for it, th in enumerate(D["thetas"][::3]):
            for pol in ("VV", "HH"):
                assert rel(s.rhs_mfie_mode(m, th, pol), D[f"Vm_{m}_{pol}"][3 * it]) < 1e-12


@pytest.mark.parametrize("name", CFIE_CASES)
def test_solve_cfie_fp64_matches_reference(pkg, name):
    D = load_golden(name)
    r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], formulation="cfie",
                                 n_modes=int(D["m_max"]), mode_tol=0.0, table_precision="double")
    assert r["formulation"] == "cfie"
    assert rel(r["amp_vv"], D["cfie_amp_vv"]) < 1e-10
    assert rel(r["amp_hh"], D["cfie_amp_hh"]) < 1e-10
    assert r["linear_residual"] < 1e-12


@pytest.mark.parametrize("name", CFIE_CASES)
def test_solve_cfie_fp32ir_within_tolerance(pkg, name):
    """CFIE with FP32 fill/LU + FP64 refinement: <= 0.01 dB and 1e-4 relative amplitude."""
    D = load_golden(name)
    r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], formulation="cfie",
                                 n_modes=int(D["m_max"]), mode_tol=0.0, table_precision="auto")
    assert r["precision"] == "fp32ir"
    for pol in ("vv", "hh"):
        assert rel(r[f"amp_{pol}"], D[f"cfie_amp_{pol}"]) < 1e-4
        assert db_err(r[f"amp_{pol}"], D[f"cfie_amp_{pol}"]) < 0.01


def test_solve_mfie_and_alpha_vs_oracle(pkg, oracle):
    """Pure MFIE and a non-default CFIE weight vs the oracle's FP64 solve."""
    D = load_golden("sphere_n24")
    M = 8
    th = D["thetas"][::2]
    for form, alpha in (("mfie", 0.5), ("cfie", 0.2)):
        want = oracle.solve_bor(D["points"], float(D["freq_hz"]), th, formulation=form, cfie_alpha=alpha,
                                n_modes=M, mode_tol=0.0)
        for tp, tol in (("double", 1e-10), ("auto", 1e-4)):
            got = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), th, formulation=form,
                                           cfie_alpha=alpha, n_modes=M, mode_tol=0.0, table_precision=tp)
            for pol in ("vv", "hh"):
                assert rel(got[f"amp_{pol}"], want[f"amp_{pol}"]) < tol, (form, tp, pol)


def test_cfie_large_body_fp32ir_vs_fp64(pkg):
    """The 600-segment cone-sphere at ka = 20 (|m| <= 25, 0.5 deg steps): the
    FP32+IR CFIE sweep stays within 1e-4 / 0.01 dB of the FP64 CFIE sweep."""
    bodies = pkg.bodies
    pts = bodies.cone_sphere_generatrix(0.5, 15.0, 600)
    k = 40.0
    f = k * 299_792_458.0 / (2 * np.pi)
    th = np.arange(0.0, 180.0 + 1e-9, 0.5)
    r32 = pkg.bor_solver.solve_bor(pts, f, th, formulation="cfie", n_modes=25, mode_tol=0.0,
                                   table_precision="auto")
    r64 = pkg.bor_solver.solve_bor(pts, f, th, formulation="cfie", n_modes=25, mode_tol=0.0,
                                   table_precision="double")
    for pol in ("vv", "hh"):
        assert rel(r32[f"amp_{pol}"], r64[f"amp_{pol}"]) < 1e-4
        assert db_err(r32[f"amp_{pol}"], r64[f"amp_{pol}"]) < 0.01
