"""Surface impedance (IBC-EFIE) and lossless penetrable bodies (PMCHWT) on
the GPU against the reference.

tests/golden/ibc_conesphere_n40.npz holds the reference's own FP64 results
(tests/golden/make_ibc_golden.py): the per-mode IBC operator additions
Z_s (M/2) + B for a tapered complex Z_s with a bare (Z_s = 0) nose, and the
full-solve amplitudes with that taper and with a scalar Z_s.  The GPU path
(ghost_bor_far_ibc, ghost_bor_near_ibc, ghost_bor_rhs_weighted) must give the
operator to 1e-11 of its largest entry, the FP64 solve to 1e-10 relative
amplitude and the FP32 + refinement solve to 1e-4 and 0.01 dB.  The far
bracket blocks and the far field with the eliminated magnetic current are
checked against the oracle, the lossless-Z_s resonance monitor against the
oracle's condition numbers, and impedance spheres against the Mie series.

tests/golden/pmchwt_sphere_n24.npz holds the reference's exterior PMCHWT
operator P and its solve_bor_dielectric amplitudes; the GPU dielectric path
(lossless media: every block from the fills above) must give P to 1e-11 and
the eps_r = 4 solve to 1e-10, the operators in a medium must equal the
oracle's, and a dielectric sphere must match the Mie series.
"""

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def D():
    return load_golden("ibc_conesphere_n40")


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def db_err(a, b):
    a, b = np.abs(np.asarray(a)) ** 2, np.abs(np.asarray(b)) ** 2
    return float(np.max(np.abs(10 * np.log10(a / b))))


def test_ibc_operator_matches_reference(pkg, D):
    """assemble_ibc_extra (far + near brackets + Z_s mass) of modes 0, 1, -4."""
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]))
    zs = D["zs_taper"]
    M = int(D["m_max"])
    for m in D["modes"]:
        m = int(m)
        err = rel(s.assemble_ibc_extra(m, M, zs[s.g.elem], zs), D[f"Zi_{m}"])
        print(f"\nmode {m}: {err:.2e}")
        assert err < 1e-11, (m, err)


def test_sample_ibc_matches_oracle(pkg, oracle):
    """Drop-in device IBC sampler (sample_ibc's argument list) vs the oracle's
    brackets, FP64."""
    import torch
    nat = pkg._native
    rng = np.random.default_rng(1)
    nr, npp, nx = 6, 13, 48
    a = [rng.uniform(0.01, 1, nr) for _ in range(4)]
    b = [rng.uniform(0.01, 1, npp) for _ in range(4)]
    xi = 2 * np.pi * np.arange(nx) / nx - np.pi
    keep = []

    def d(v):
        t = torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device="cuda")
        keep.append(t)
        return t

    outs = [torch.empty((nr, npp, nx), dtype=torch.complex128, device="cuda") for _ in range(4)]
    args = [nat.ptr(d(v)) for v in a] + [nat.ptr(d(v)) for v in b]
    nat.call("ghost_bor_sample_ibc", nr, npp, nx, *args, 7.5, nat.ptr(d(np.cos(xi))),
             nat.ptr(d(np.sin(xi))), *[nat.ptr(o) for o in outs], nat.stream_handle())
    one = np.ones((nr, npp))
    F = oracle._ibc_bracket_grid(*[(v[:, None] * one).ravel() for v in a],
                                 *[(v[None, :] * one).ravel() for v in b], 7.5,
                                 np.broadcast_to(xi, (nr * npp, nx)))
    for o, f in zip(outs, F):
        assert rel(o.cpu().numpy(), f.reshape(nr, npp, nx)) < 1e-13


def test_ibc_far_bracket_blocks(pkg, oracle, D):
    """Streamed IBC far blocks with Z_s in the source weights (FP64 and FP32
    transforms) vs the oracle's, every mode -M..M."""
    M = int(D["m_max"])
    zs = D["zs_taper"]
    o = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    o.build_far(M, efie=False, ibc_zs_pt=zs[o.geo.elem])
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]))
    for dtype, tol in ((np.complex128, 1e-12), (np.complex64, 1e-5)):
        s.enable_streaming(M, efie=False, ibc_zs_pt=zs[s.g.elem], single_blocks=dtype == np.complex64)
        for m in range(-M, M + 1):
            got = s._stream.bracket_blocks("ibc", m)
            want = [o.Bb[uv, m + M] for uv in range(4)]
            scale = max(np.max(np.abs(w)) for w in want)
            err = max(np.max(np.abs(g - w)) for g, w in zip(got, want)) / scale
            assert err < tol, (dtype, m, err)


@pytest.mark.parametrize("tag", ["taper", "scalar"])
@pytest.mark.parametrize("precision,rel_tol,db_tol", [("double", 1e-10, 1e-6), ("auto", 1e-4, 0.01)])
def test_ibc_solve_matches_reference(pkg, D, tag, precision, rel_tol, db_tol):
    zs = D["zs_taper"] if tag == "taper" else 120.0 - 80.0j
    r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], formulation="efie",
                                 zs=zs, n_modes=int(D["m_max"]), mode_tol=0.0, table_precision=precision)
    for pol in ("vv", "hh"):
        a, b = r[f"amp_{pol}"], D[f"amp_{pol}_{tag}"]
        print(f"\n{tag} {precision} {pol}: rel {rel(a, b):.2e}, dB {db_err(a, b):.2e}")
        assert rel(a, b) < rel_tol
        assert db_err(a, b) < db_tol
    assert "max_cond" not in r          # lossy Z_s: no resonance monitor


def test_ibc_farfield_mode_matches_oracle(pkg, oracle, D):
    """Far field of J plus the eliminated M = -Z_s n x J by reciprocity
    (V_E - V_H^Zs from ghost_bor_rhs_weighted) vs the oracle's projection."""
    zs = D["zs_taper"]
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]))
    o = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    rng = np.random.default_rng(4)
    for m in (0, 1, -3):
        for th in (20.0, 90.0, 151.0):
            x = rng.standard_normal(2 * s.Nn) + 1j * rng.standard_normal(2 * s.Nn)
            got = s.farfield_mode(m, x, th, zs_pt=zs[s.g.elem])
            fth, fph = o.farfield(m, x[None, :], [th], zs_pt=zs[o.geo.elem])
            want = np.array([fth[0], fph[0]])
            assert np.max(np.abs(np.array(got) - want)) <= 1e-12 * np.max(np.abs(want)), (m, th)


@pytest.mark.parametrize("precision,tol", [("double", 1e-6), ("auto", 1e-2)])
def test_lossless_ibc_resonance_monitor(pkg, oracle, D, precision, tol):
    """A closed body with a purely reactive Z_s on the EFIE: the warning and the
    per-mode condition numbers (max, median over the modes used) of the
    reference's monitor, against np.linalg.cond of the oracle's systems."""
    zs = -50j
    M = int(D["m_max"])
    r = pkg.bor_solver.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"], formulation="efie",
                                 zs=zs, n_modes=M, mode_tol=0.0, table_precision=precision)
    assert any("lossless" in w for w in r["warnings"])
    o = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    ze = np.full(o.geo.ne, zs)
    o.prepare(M, efie=True, mfie=False, workers=4, ibc_zs_pt=ze[o.geo.elem])
    conds = []
    for m in range(M + 1):
        A = o.assemble_efie(m, M) + o.assemble_ibc_extra(m, M, ze[o.geo.elem], ze)
        keep = o.basis_mask(m)
        conds.append(np.linalg.cond(A[np.ix_(keep, keep)]))
    print(f"\n{precision}: max_cond {r['max_cond']:.6e} vs {max(conds):.6e}, "
          f"median {r['median_cond']:.6e} vs {np.median(conds):.6e}")
    assert abs(r["max_cond"] - max(conds)) <= tol * max(conds)
    assert abs(r["median_cond"] - np.median(conds)) <= tol * np.median(conds)


@pytest.mark.parametrize("a,f,zs", [(0.5, 3e8, 50 - 20j), (0.3, 1e9, 100 + 100j)])
def test_impedance_sphere_matches_mie(pkg, a, f, zs):
    """Backscatter of a 120-segment impedance sphere vs the impedance-sphere
    Mie series (oracle.mie, pinned to the reference's): the mesh's own
    discretisation error is 0.0024 and 0.0063 dB for these two cases."""
    from oracle import mie
    pts = pkg.bodies.sphere_generatrix(a, 120)
    want = mie.sigma_impedance_sphere(a, f, zs)
    for precision in ("double", "auto"):
        r = pkg.bor_solver.solve_bor(pts, f, [0.0, 60.0, 120.0], zs=zs, mode_tol=0.0,
                                     table_precision=precision)
        s = np.array(r["sigma_vv"] + r["sigma_hh"])
        err = float(np.max(np.abs(10 * np.log10(s / want))))
        print(f"\n{precision}: {err:.4f} dB")
        assert err < 0.01, (precision, err)


# ---------------------------------------------------------------------------
# lossless penetrable bodies (PMCHWT)
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def P24():
    return load_golden("pmchwt_sphere_n24")


def test_pmchwt_P_matches_reference(pkg, P24):
    """The exterior rotated principal-value operator (unit-weight IBC brackets
    without mass term, columns remapped) of modes 0 and 2."""
    s = pkg.bor_solver.BorPecSolver(P24["points"], float(P24["freq_hz"]))
    M = int(P24["m_max"])
    for m in P24["modes"]:
        err = rel(s.assemble_pmchwt_P(int(m), M), P24[f"Pe_{int(m)}"])
        print(f"\nP_e mode {int(m)}: {err:.2e}")
        assert err < 1e-11, (int(m), err)


def test_operators_in_a_medium_match_oracle(pkg, oracle, P24):
    """T and P of a lossless medium (eps_r = 4): the generatrix at f n with the
    medium's eta, vs the oracle's complex-medium solver."""
    M = int(P24["m_max"])
    s = pkg.bor_solver.BorPecSolver(P24["points"], float(P24["freq_hz"]), medium=(4.0, 1.0))
    o = oracle.OracleSolver(P24["points"], float(P24["freq_hz"]), medium=(4.0, 1.0))
    o.prepare(M, efie=True, workers=4, ibc_zs_pt=np.ones(o.geo.P))
    for m in (0, 2, -3):
        assert rel(s.assemble_mode(m, M), o.assemble_efie(m, M)) < 1e-11, m
        assert rel(s.assemble_pmchwt_P(m, M), o.pmchwt_P(m, M)) < 1e-11, m


def test_dielectric_solve_matches_reference(pkg, P24):
    r = pkg.bor_solver.solve_bor_dielectric(P24["points"], float(P24["freq_hz"]), P24["thetas"], 4.0, 1.0,
                                            n_modes=int(P24["m_max"]), mode_tol=0.0)
    for pol in ("vv", "hh"):
        a, b = r[f"amp_{pol}"], P24[f"amp_{pol}_1"]
        print(f"\n{pol}: rel {rel(a, b):.2e}, dB {db_err(a, b):.2e}")
        assert rel(a, b) < 1e-10
    assert r["linear_residual"] < 1e-10


def test_dielectric_sphere_matches_mie(pkg):
    """A 60-segment eps_r = 2.5 sphere, ka = pi: the oracle's own error against
    the Mie series is 0.0085 dB at this mesh."""
    from oracle import mie
    a, f, eps = 0.5, 3e8, 2.5
    r = pkg.bor_solver.solve_bor_dielectric(pkg.bodies.sphere_generatrix(a, 60), f, [0.0, 60.0, 120.0],
                                            eps, 1.0, mode_tol=0.0)
    want = mie.sigma_dielectric_sphere(a, eps, 1.0, f)
    s = np.array(r["sigma_vv"] + r["sigma_hh"])
    err = float(np.max(np.abs(10 * np.log10(s / want))))
    print(f"\n{err:.4f} dB")
    assert err < 0.02


# lossy media: the complex-wave-number fills of the interior

@pytest.mark.parametrize("case", [0, 2])
def test_lossy_dielectric_solve_matches_reference(pkg, P24, case):
    """eps_r = 2.5 - 0.2j; eps_r = 2 - 0.1j with mu_r = 1.5 - 0.2j."""
    eps, mu = (complex(x) for x in P24["media"][case])
    r = pkg.bor_solver.solve_bor_dielectric(P24["points"], float(P24["freq_hz"]), P24["thetas"], eps, mu,
                                            n_modes=int(P24["m_max"]), mode_tol=0.0)
    for pol in ("vv", "hh"):
        a, b = r[f"amp_{pol}"], P24[f"amp_{pol}_{case}"]
        print(f"\n{case} {pol}: rel {rel(a, b):.2e}")
        assert rel(a, b) < 1e-10


def test_lossy_medium_operators_match_reference(pkg, P24):
    """T_i and P_i of the eps_r = 2.5 - 0.2j medium, modes 0 and 2, against the
    reference's BorPecSolver(medium=...)."""
    M = int(P24["m_max"])
    s = pkg.bor_solver.BorPecSolver(P24["points"], float(P24["freq_hz"]),
                                    medium=tuple(complex(x) for x in P24["media"][0]))
    for m in P24["modes"]:
        m = int(m)
        assert rel(s.assemble_mode(m, M), P24[f"Ti_{m}"]) < 1e-11, m
        assert rel(s.assemble_pmchwt_P(m, M), P24[f"Pi_{m}"]) < 1e-11, m


def test_lossy_dielectric_sphere_matches_mie(pkg):
    """A 60-segment eps_r = 4 - 0.5j sphere (a = 0.3 m, 1 GHz): the oracle's own
    error against the Mie series is 0.016 dB at this mesh."""
    from oracle import mie
    a, f, eps = 0.3, 1e9, 4.0 - 0.5j
    r = pkg.bor_solver.solve_bor_dielectric(pkg.bodies.sphere_generatrix(a, 60), f, [0.0, 60.0, 120.0],
                                            eps, 1.0, mode_tol=0.0)
    want = mie.sigma_dielectric_sphere(a, eps, 1.0, f)
    s = np.array(r["sigma_vv"] + r["sigma_hh"])
    err = float(np.max(np.abs(10 * np.log10(s / want))))
    print(f"\n{err:.4f} dB")
    assert err < 0.03
