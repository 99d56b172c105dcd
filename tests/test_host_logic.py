"""Host logic of the GPU engine checked on the CPU oracle: the +-m folding
and reciprocity identities the engine relies on, and the truncation replay."""
import numpy as np
import pytest

from conftest import load_golden


def test_mode_symmetry_and_reciprocity(oracle):
    D = load_golden("conesphere_n40")
    s = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    M = int(D["m_max"])
    s.prepare(M, efie=True)
    Nn = s.geo.Nn
    d = np.concatenate([np.ones(Nn), -np.ones(Nn)])
    th = D["thetas"]
    c = -1j * s.k * oracle.ETA0 / (4 * np.pi)
    for m in (1, 3, 8):
        Zp, Zm = s.assemble_efie(m, M), s.assemble_efie(-m, M)
        assert np.max(np.abs(Zm - d[:, None] * Zp * d[None, :])) <= 1e-13 * np.max(np.abs(Zp))
        Vv, Vh = s.rhs_efie(m, th, "VV"), s.rhs_efie(m, th, "HH")
        Vvm, Vhm = s.rhs_efie(-m, th, "VV"), s.rhs_efie(-m, th, "HH")
        assert np.allclose(Vvm, Vv * d, rtol=0, atol=1e-13 * np.abs(Vv).max())
        assert np.allclose(Vhm, -Vh * d, rtol=0, atol=1e-13 * np.abs(Vh).max())
        rng = np.random.default_rng(m)
        x = rng.standard_normal((len(th), 2 * Nn)) + 1j * rng.standard_normal((len(th), 2 * Nn))
        fth, fph = s.farfield(m, x, th)
        assert np.allclose(fth, c * np.sum(d * Vv * x, axis=1), rtol=1e-12, atol=0)
        assert np.allclose(fph, -c * np.sum(d * Vh * x, axis=1), rtol=1e-12, atol=0)


def test_truncation_replay(pkg, oracle):
    """replay_truncation reproduces the reference loop's modes_used and F."""
    eng = pytest.importorskip("importlib").import_module("20260722_ghost_gb300.engine")
    rng = np.random.default_rng(0)
    dF = rng.standard_normal((12, 2, 5)) + 1j * rng.standard_normal((12, 2, 5))
    dF *= np.exp(-np.arange(12))[:, None, None]
    for tol in (0.0, 1e-6, 1e-3, 1e-1):
        F, used = eng.replay_truncation(dF, tol)
        Fr = np.zeros((2, 5), complex)
        quiet, used_r = 0, 0
        for am in range(12):
            Fr += dF[am]
            used_r = am
            if np.max(np.abs(dF[am])) < tol * max(np.max(np.abs(Fr)), 1e-30):
                quiet += 1
                if quiet >= 2:
                    break
            else:
                quiet = 0
        assert used == used_r and np.array_equal(F, Fr)


def test_adjoint_identity_on_oracle(pkg, oracle):
    """The gradient formula of the adjoint module, dF = s c [2 (Dx)^T dV -
    (Dx)^T dZ x] (reciprocity adjoint y = D x), against a central difference
    of the oracle's far field for a B-spline body; and Z^T = D Z D up to the
    quadrature's symmetry."""
    O = oracle
    bodies = pkg.bodies
    radii = np.random.default_rng(0).uniform(0.3, 0.6, 6)
    N, k, M, m = 30, 6.0, 3, 2
    f = k * O.C0 / (2 * np.pi)
    th = np.array([35.0, 50.0])

    def build(r):
        s = O.OracleSolver(bodies.bspline_body(r, N)[0], f)
        s.build_far(M, efie=True)
        return s

    s0 = build(radii)
    Nn = s0.geo.Nn
    D = np.concatenate([np.ones(Nn), -np.ones(Nn)])
    Z = s0.assemble_efie(m, M)
    assert np.max(np.abs(Z.T - D[:, None] * Z * D[None, :])) < 1e-4 * np.max(np.abs(Z))
    mask = s0.basis_mask(m)
    c = -1j * k * O.ETA0 / (4 * np.pi)

    def field(s):
        A = s.assemble_efie(m, M)[np.ix_(mask, mask)]
        V = s.rhs_efie(m, th, "HH")[:, mask].T
        x = np.linalg.solve(A, V)
        return -c * np.sum(D[mask][:, None] * V * x, axis=0), A, V, x

    _, A0, V0, x0 = field(s0)
    h, j = 1e-5, 2
    rp, rm = radii.copy(), radii.copy()
    rp[j] += h
    rm[j] -= h
    Fp, Ap, Vp, _ = field(build(rp))
    Fm, Am, Vm, _ = field(build(rm))
    dZ, dV = (Ap - Am) / (2 * h), (Vp - Vm) / (2 * h)
    Dm = D[mask][:, None]
    Dx = Dm * x0
    fd = (Fp - Fm) / (2 * h)
    # reciprocity adjoint y = D x (exact only for a symmetric quadrature)
    adj_sym = -c * (2 * np.sum(Dx * dV, axis=0) - np.sum(Dx * (dZ @ x0), axis=0))
    assert np.max(np.abs(adj_sym - fd)) < 1e-4 * np.max(np.abs(fd))
    # the adjoint module's y = D x + D A^-1 D s, s = D V - A^T D x, against the
    # exact adjoint solution A^T y = D V and the central difference
    y_exact = np.linalg.solve(A0.T, Dm * V0)
    s_ = Dm * V0 - A0.T @ Dx
    y = Dx + Dm * np.linalg.solve(A0, Dm * s_)
    assert np.max(np.abs(y - y_exact)) < 1e-7 * np.max(np.abs(y_exact))
    adj = -c * (np.sum(Dx * dV, axis=0) + np.sum(y * (dV - dZ @ x0), axis=0))
    assert np.max(np.abs(adj - fd)) < 1e-6 * np.max(np.abs(fd))


def test_mass_blocks_match_oracle(pkg, oracle):
    """BorPecSolver.mass_blocks (geometry only) = the oracle's mass term, plain
    and weighted per Gauss point (the Z_s mass of an impedance surface)."""
    import importlib
    bs = importlib.import_module("20260722_ghost_gb300.bor_solver")
    D = load_golden("conesphere_n40")
    s = bs.BorPecSolver(D["points"], float(D["freq_hz"]))
    o = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    w = np.linspace(50.0, 300.0, s.P) - 20.0j
    for weight in (None, w):
        got, want = s.mass_blocks(weight), o.mass(weight)
        assert np.max(np.abs(got - want)) <= 1e-14 * np.max(np.abs(want))


@pytest.mark.parametrize("dtype", ["complex128", "complex64", "float64", "int32", "uint8"])
def test_guard_band_helper_detects_margin_writes(dtype):
    """The guard-band buffers of the GPU stage test, on CPU tensors: writes
    inside the view keep check() true, one element past either end fails it."""
    import torch
    from guard_bands import guarded
    dt = getattr(torch, dtype)
    v, chk = guarded((3, 5, 7), dt, "cpu")
    assert tuple(v.shape) == (3, 5, 7) and v.is_contiguous() and chk()
    assert (v.data_ptr() - chk.base.data_ptr()) % 256 == 0
    v.fill_(1)
    assert chk()
    for idx in (chk.pad - 1, chk.pad + v.numel()):
        w, chk2 = guarded((3, 5, 7), dt, "cpu")
        chk2.base[idx] = 1
        assert not chk2(), idx


def test_drop_in_arguments_and_no_cpu_fallback(pkg):
    """solve_bor rejects bad arguments as the reference does (before any device
    work) and, with valid arguments and no CUDA device, raises instead of
    computing anything on the host."""
    import importlib
    import torch
    bs = importlib.import_module("20260722_ghost_gb300.bor_solver")
    pts = pkg.bodies.sphere_generatrix(1.0, 12)
    f = 3e8
    with pytest.raises(ValueError):
        bs.solve_bor(pts, f, [0.0], formulation="pmchwt")
    with pytest.raises(ValueError):
        bs.solve_bor(pts, f, [0.0], table_precision="half")
    with pytest.raises(ValueError):
        bs.solve_bor(pts, f, [0.0], assembly="fmm")
    with pytest.raises(ValueError):
        bs.solve_bor_batch([{"points": pts, "freq_hz": f}], [0.0], table_precision="quad")

    def abort():
        raise InterruptedError("cancelled")

    with pytest.raises(InterruptedError):
        bs.solve_bor(pts, f, [0.0], check_abort=abort)
    with pytest.raises(NotImplementedError):
        bs.BorPecSolver(pts, f, medium=(-2.0, 1.0))              # evanescent: Re m = 0
    with pytest.raises(NotImplementedError):
        bs.solve_bor_dielectric(pts, f, [0.0], -2.0, 1.0)
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            bs.solve_bor_dielectric(pts, f, [0.0], 2.0, 1.0)
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            bs.solve_bor_dielectric(pts, f, [0.0], 2.0 - 0.1j, 1.0)
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            bs.solve_bor(pts, f, [0.0, 90.0])
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            bs.solve_bor(pts, f, [0.0], zs=50.0)
        with pytest.raises(RuntimeError, match="no CPU fallback"):
            bs.BorPecSolver(pts, f).assemble_mode(0, 2)


def test_non_finite_inputs_rejected_before_device_work(pkg):
    """NaN / inf nodes or angles and non-positive frequencies never reach a
    kernel: BorGpuProblem raises ValueError before touching the device."""
    import importlib
    eng = importlib.import_module("20260722_ghost_gb300.engine")
    pts = pkg.bodies.sphere_generatrix(1.0, 12)
    bad = pts.copy()
    bad[3, 0] = np.nan
    for args in ((bad, 3e8, [0.0]), (pts, 3e8, [0.0, np.inf]), (pts, float("nan"), [0.0]),
                 (pts, -1.0, [0.0]), (pts, 0.0, [0.0])):
        with pytest.raises(ValueError):
            eng.BorGpuProblem(*args)


def test_mode_runs_groups_live_modes(pkg):
    """The refinement corrects only the modes still above the floor, as runs of
    consecutive modes (one batched launch per run)."""
    runs = pkg.engine.mode_runs
    assert runs(np.array([1, 1, 0, 1, 0, 0, 1, 1, 1], bool)) == [(0, 2), (3, 4), (6, 9)]
    assert runs(np.zeros(5, bool)) == []
    assert runs(np.ones(4, bool)) == [(0, 4)]
    rng = np.random.default_rng(3)
    for _ in range(50):
        live = rng.random(rng.integers(1, 40)) < 0.5
        got = np.zeros_like(live)
        for a, b in runs(live):
            assert a < b and not got[a:b].any()
            got[a:b] = True
        assert np.array_equal(got, live)


def test_refine_for_currents_settings(pkg):
    """The surface-current refinement: every correction updated with exact
    products, each mode refined to 1e-11 of its right-hand side."""
    eng = pkg.engine
    prob = object.__new__(eng.BorGpuProblem)
    prob.exact_update_iters, prob.refine_floor = 1, 2e-9
    prob.refine_for_currents()
    assert prob.exact_update_iters is None and prob.refine_floor == 1e-11


def test_far_blocks_mirror_relation(oracle):
    """The relation the tensor-core far fill writes the mirror pair with: for
    node pairs reached only by far element pairs (|i - j| >= 3), the EFIE
    operator of every mode satisfies Z_tt^T = Z_tt, Z_ff^T = Z_ff and
    Z_tf^T = -Z_ft, so the blocks of (f, e) are b0, -b2, -b1, b3 of (e, f)."""
    D = load_golden("conesphere_n40")
    s = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    M = int(D["m_max"])
    s.prepare(M, efie=True)
    Nn = s.geo.Nn
    far = np.abs(np.arange(Nn)[:, None] - np.arange(Nn)[None, :]) >= 3
    for m in (0, 1, 4, M):
        Z = s.assemble_efie(m, M)
        tt, tf, ft, ff = Z[:Nn, :Nn], Z[:Nn, Nn:], Z[Nn:, :Nn], Z[Nn:, Nn:]
        top = np.max(np.abs(Z))
        assert np.max(np.abs((tt - tt.T)[far])) <= 1e-13 * top, m
        assert np.max(np.abs((ff - ff.T)[far])) <= 1e-13 * top, m
        assert np.max(np.abs((tf + ft.T)[far])) <= 1e-13 * top, m


def test_step_g_chebyshev_recurrence_covers_every_order():
    """The grouped near kernel's order mapping: lane q of G starts the step-G
    recurrence c_{n+G} = 2 cos(G xi) c_n - c_{n-G} from (cos((G - q) xi),
    cos(q xi)) (cos((q - G) xi) = cos((G - q) xi)) and visits n = q, q + G, ...;
    every order is visited once and gets cos(n xi)."""
    rng = np.random.default_rng(4)
    for G in (2, 4, 8, 16):
        Mp = 16 * G - 3
        xi = rng.uniform(0.0, np.pi, 64)
        T = np.cos(np.arange(G + 1)[:, None] * xi[None, :])        # the evaluating lane's ladder
        got = np.full((Mp, xi.size), np.nan)
        for q in range(G):
            cm, c0, t = T[G - q], T[q], 2.0 * T[G]
            for i in range((Mp + G - 1) // G):
                n = q + i * G
                if n < Mp:
                    assert np.all(np.isnan(got[n]))
                    got[n] = c0
                cm, c0 = c0, t * c0 - cm
        assert not np.any(np.isnan(got))
        np.testing.assert_allclose(got, np.cos(np.arange(Mp)[:, None] * xi[None, :]), rtol=0, atol=1e-11)
