"""GPU kernels through the C ABI against the CPU oracle / reference goldens."""
import math

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def test_sample_g_and_mfie(pkg, oracle, torch):
    """Drop-in device samplers vs the oracle's C restatement (bit-level formulas, FP64)."""
    nat = pkg._native
    rng = np.random.default_rng(1)
    nr, npp, nx = 6, 13, 48
    a = [rng.uniform(0.01, 1, nr) for _ in range(4)]
    b = [rng.uniform(0.01, 1, npp) for _ in range(4)]
    xi = 2 * np.pi * np.arange(nx) / nx - np.pi
    s2 = np.sin(0.5 * xi) ** 2
    keep = []          # device inputs must outlive the asynchronous launches

    def d(v):
        t = torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device="cuda")
        keep.append(t)
        return t

    out = torch.empty((nr, npp, nx), dtype=torch.complex128, device="cuda")
    nat.call("ghost_bor_sample_g", nr, npp, nx, nat.ptr(d(a[0])), nat.ptr(d(a[1])), nat.ptr(d(b[0])),
             nat.ptr(d(b[1])), 7.5, nat.ptr(d(s2)), nat.ptr(out), nat.stream_handle())
    dR = (a[0][:, None] - b[0][None, :]) ** 2 + (a[1][:, None] - b[1][None, :]) ** 2
    R = np.sqrt(dR[..., None] + 4 * (a[0][:, None] * b[0][None, :])[..., None] * s2)
    assert rel(out.cpu().numpy(), np.exp(-7.5j * R) / (4 * np.pi * R)) < 1e-14
    outs = [torch.empty((nr, npp, nx), dtype=torch.complex128, device="cuda") for _ in range(4)]
    args = [nat.ptr(d(v)) for v in a] + [nat.ptr(d(v)) for v in b]
    nat.call("ghost_bor_sample_mfie", nr, npp, nx, *args, 7.5, nat.ptr(d(np.cos(xi))),
             nat.ptr(d(np.sin(xi))), *[nat.ptr(o) for o in outs], nat.stream_handle())
    one = np.ones((nr, npp))
    F = oracle._mfie_bracket_grid(
        (a[0][:, None] * one).ravel(), (a[1][:, None] * one).ravel(), (a[2][:, None] * one).ravel(),
        (a[3][:, None] * one).ravel(), (b[0][None, :] * one).ravel(), (b[1][None, :] * one).ravel(),
        (b[2][None, :] * one).ravel(), (b[3][None, :] * one).ravel(), 7.5,
        np.broadcast_to(xi, (nr * npp, nx)))
    for o, f in zip(outs, F):
        assert rel(o.cpu().numpy(), f.reshape(nr, npp, nx)) < 1e-13


@pytest.mark.parametrize("name", ["sphere_n24", "conesphere_n40", "openshell_n20"])
def test_far_blocks(pkg, oracle, name):
    """Fused far fill (FP64 and FP32) vs the oracle's streamed far blocks."""
    D = load_golden(name)
    M = int(D["m_max"])
    o = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    o.build_far(M, efie=True)
    bs = pkg.bor_solver
    s = bs.BorPecSolver(D["points"], float(D["freq_hz"]))
    for dtype, tol in ((np.complex128, 1e-12), (np.complex64, 2e-5)):
        s.enable_streaming(M, single_blocks=dtype == np.complex64)
        for m in list(range(M + 1)) + [-1, -M]:
            got = s._stream.efie_blocks(m)
            want = o.efie_far_blocks(m)
            scale = max(np.max(np.abs(w)) for w in want)
            err = max(np.max(np.abs(g - w)) for g, w in zip(got, want)) / scale
            assert err < tol, (dtype, m, err)


def test_far_fill_wide_order_rows(pkg, torch):
    """|m| <= 90: the FP32 far fill covers every order in one launch row (two
    element pairs and eight order groups per CTA), the FP64 fill in two rows;
    both agree to the FP32 fill's accuracy on every mode."""
    bodies = pkg.bodies
    eng = pkg.engine
    nat = pkg._native
    pts = bodies.cone_sphere_generatrix(0.5, 15.0, 120)
    prob = eng.BorGpuProblem(pts, 60.0 * 299792458.0 / (2 * math.pi), np.array([0.0, 90.0]), m_max=90)
    Mb, n = prob.m_max + 1, prob.n
    st = nat.stream_handle()
    Z64 = torch.zeros((Mb, n, n), dtype=torch.complex128, device="cuda")
    Z32 = torch.zeros_like(Z64)
    prob.fill_far(Z64, nat.F64, 1.0 + 0.0j, st)
    prob.fill_far(Z32, nat.F32, 1.0 + 0.0j, st)
    torch.cuda.synchronize()
    top = Z64.abs().max().item()
    for m in range(Mb):
        scale = Z64[m].abs().max().item()
        err = (Z32[m] - Z64[m]).abs().max().item()
        assert scale > 0.0
        assert err < 2e-5 * top and err < 1e-3 * scale, (m, err / scale)


@pytest.mark.parametrize("m_max,n_seg,k", [(20, 60, 20.0), (50, 80, 40.0), (90, 120, 60.0), (200, 60, 60.0)])
def test_far_fill_tensor_cores(pkg, torch, m_max, n_seg, k):
    """The tensor-core FP32 far fill (exact digit transform) against the FP64
    fill on every mode: tiles of 32, 64 and 128 orders, one and two launch
    rows (|m| = 200), 129..513 azimuth samples; it is far closer to FP64 than
    the SIMT FP32 transform."""
    eng = pkg.engine
    nat = pkg._native
    pts = pkg.bodies.cone_sphere_generatrix(0.5, 15.0, n_seg)
    prob = eng.BorGpuProblem(pts, k * 299792458.0 / (2 * math.pi), np.array([0.0, 90.0]), m_max=m_max)
    Mb, n = prob.m_max + 1, prob.n
    st = nat.stream_handle()
    Z64 = torch.zeros((Mb, n, n), dtype=torch.complex128, device="cuda")
    Ztc = torch.zeros_like(Z64)
    Zs = torch.zeros_like(Z64)
    prob.fill_far(Z64, nat.F64, 1.0 + 0.0j, st)
    prob.far_tc = True
    prob.fill_far(Ztc, nat.F32, 1.0 + 0.0j, st)
    prob.far_tc = False
    prob.fill_far(Zs, nat.F32, 1.0 + 0.0j, st)
    torch.cuda.synchronize()
    prob.check_far_status()
    top = Z64.abs().max().item()
    e_tc = (Ztc - Z64).abs().amax(dim=(1, 2)).cpu().numpy() / top
    e_simt = (Zs - Z64).abs().amax(dim=(1, 2)).cpu().numpy() / top
    print(f"\nM={m_max} N={n_seg} k={k} n_xi={prob.n_xi}: max rel err tc {e_tc.max():.3e} simt {e_simt.max():.3e}")
    assert np.all(np.isfinite(e_tc))
    assert e_tc.max() < 2e-6, e_tc
    assert e_tc.max() < e_simt.max(), (e_tc.max(), e_simt.max())


@pytest.mark.parametrize("name", ["sphere_n24", "conesphere_n40", "openshell_n20"])
def test_full_operator_and_excitation(pkg, name):
    """assemble_mode (far + near), rhs_mode and farfield_mode vs the reference goldens."""
    D = load_golden(name)
    M = int(D["m_max"])
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]))
    s.prepare_operators(M)
    for m in D["modes"]:
        m = int(m)
        assert rel(s.assemble_mode(m, M), D[f"Ze_{m}"]) < 1e-12, m
        np.testing.assert_array_equal(s.basis_mask(m), D[f"mask_{m}"])
        for it, th in enumerate(D["thetas"][::3]):
            for pol in ("VV", "HH"):
                assert rel(s.rhs_mode(m, th, pol), D[f"Ve_{m}_{pol}"][3 * it]) < 1e-12
        x = D[f"ffx_{m}"]
        ff = np.array([s.farfield_mode(m, x, th) for th in D["thetas"][::4]])
        assert rel(ff, D[f"ff_{m}"][::4]) < 1e-12


@pytest.mark.parametrize("prec,tol,tc", [("f64", 1e-11, False), ("f32", 5e-4, False), ("f32", 5e-4, True)])
def test_batched_lu(pkg, torch, prec, tol, tc):
    """ghost_bor_getrf / getrs vs numpy on random complex systems, including a
    size that is not a multiple of the panel width and pivoting-heavy rows."""
    nat = pkg._native
    rng = np.random.default_rng(5)
    batch, n, nrhs = 3, 173, 37
    A = rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))
    A[:, 0, :] *= 1e-3                          # force pivoting
    B = rng.standard_normal((batch, n, nrhs)) + 1j * rng.standard_normal((batch, n, nrhs))
    X_ref = np.linalg.solve(A, B)
    dt = torch.complex128 if prec == "f64" else torch.complex64
    p = nat.F64 if prec == "f64" else nat.F32
    dA = torch.as_tensor(A, device="cuda").to(dt).contiguous()
    dB = torch.as_tensor(B, device="cuda").to(dt).contiguous()
    ipiv = torch.empty((batch, n), dtype=torch.int32, device="cuda")
    info = torch.empty((batch,), dtype=torch.int32, device="cuda")
    st = nat.stream_handle()
    lib = nat.load()
    wf = torch.empty(max(1, int(lib.ghost_bor_getrf_workspace(p, batch, n))), dtype=torch.uint8, device="cuda")
    ws = torch.empty(max(1, int(lib.ghost_bor_getrs_workspace(p, batch, n, nrhs))), dtype=torch.uint8,
                     device="cuda")
    nat.call("ghost_bor_getrf", p, batch, n, nat.ptr(dA), n, n * n, nat.ptr(ipiv), nat.ptr(info),
             nat.ptr(wf) if tc else 0, st)
    nat.call("ghost_bor_getrs", p, batch, n, nrhs, nat.ptr(dA), n, n * n, nat.ptr(ipiv), nat.ptr(dB),
             nrhs, n * nrhs, nat.ptr(ws) if tc else 0, st)
    if tc:
        assert int(wf[:4].view(torch.int32)[0].cpu()) == 0 and int(ws[:4].view(torch.int32)[0].cpu()) == 0
    X = dB.cpu().numpy()
    assert np.all(info.cpu().numpy() == 0)
    assert rel(X, X_ref) < tol
    # partial pivoting with the |re| + |im| rule: |l| <= sqrt(2) |pivot| / |pivot|
    LU = dA.cpu().numpy()
    L = np.tril(LU, -1)
    assert np.max(np.abs(L)) <= math.sqrt(2.0) * (1.0 + 1e-5)


def test_singular_pivot_reported(pkg, torch):
    nat = pkg._native
    n = 70
    A = np.eye(n, dtype=np.complex128)
    A[40, 40] = 0.0
    dA = torch.as_tensor(A[None], device="cuda").contiguous()
    ipiv = torch.empty((1, n), dtype=torch.int32, device="cuda")
    info = torch.empty((1,), dtype=torch.int32, device="cuda")
    nat.call("ghost_bor_getrf", nat.F64, 1, n, nat.ptr(dA), n, n * n, nat.ptr(ipiv), nat.ptr(info), 0,
             nat.stream_handle())
    assert int(info.cpu()[0]) == 41


@pytest.mark.parametrize("n", [700, 1500, 2900, 3200, 6002])
def test_blocked_panel_lu_sizes(pkg, torch, n):
    """The FP32 LU with the register-blocked panel (256 threads holding 4, 8,
    12, 16 or 24 rows each, sub-blocks of 4 or 2 columns) on the
    tensor-core path: solution vs numpy, the pivoting bound, and the pivots of
    an FP64 LU of the same matrix where no near-tie decides them."""
    nat = pkg._native
    rng = np.random.default_rng(n)
    batch, nrhs = 2, 8
    A = rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))
    A[:, : n // 3, :] *= 1e-2                   # pivots come from below
    B = rng.standard_normal((batch, n, nrhs)) + 1j * rng.standard_normal((batch, n, nrhs))
    X_ref = np.linalg.solve(A, B)
    p = nat.F32
    dA = torch.as_tensor(A, device="cuda").to(torch.complex64).contiguous()
    dB = torch.as_tensor(B, device="cuda").to(torch.complex64).contiguous()
    ipiv = torch.empty((batch, n), dtype=torch.int32, device="cuda")
    info = torch.empty((batch,), dtype=torch.int32, device="cuda")
    st = nat.stream_handle()
    lib = nat.load()
    wf = torch.empty(int(lib.ghost_bor_getrf_workspace(p, batch, n)), dtype=torch.uint8, device="cuda")
    ws = torch.empty(int(lib.ghost_bor_getrs_workspace(p, batch, n, nrhs)), dtype=torch.uint8, device="cuda")
    nat.call("ghost_bor_getrf", p, batch, n, nat.ptr(dA), n, n * n, nat.ptr(ipiv), nat.ptr(info), nat.ptr(wf), st)
    nat.call("ghost_bor_getrs", p, batch, n, nrhs, nat.ptr(dA), n, n * n, nat.ptr(ipiv), nat.ptr(dB),
             nrhs, n * nrhs, nat.ptr(ws), st)
    torch.cuda.synchronize()
    assert int(wf[:4].view(torch.int32)[0].cpu()) == 0 and int(ws[:4].view(torch.int32)[0].cpu()) == 0
    assert np.all(info.cpu().numpy() == 0)
    X = dB.cpu().numpy()
    # FP32 LU of a random n x n system: error ~ n eps_32 kappa
    assert rel(X, X_ref) < 2e-2, rel(X, X_ref)
    L = np.tril(dA.cpu().numpy(), -1)
    assert np.max(np.abs(L)) <= math.sqrt(2.0) * (1.0 + 1e-5)
    # the first panel's pivots equal those of the FP64 LU (no near-ties at this scale)
    dA64 = torch.as_tensor(A, device="cuda").contiguous()
    ip64 = torch.empty_like(ipiv)
    nat.call("ghost_bor_getrf", nat.F64, batch, n, nat.ptr(dA64), n, n * n, nat.ptr(ip64), nat.ptr(info), 0, st)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ipiv.cpu().numpy()[:, :16], ip64.cpu().numpy()[:, :16])


def test_singular_pivot_reported_blocked_panel(pkg, torch):
    nat = pkg._native
    n = 300
    A = np.eye(n, dtype=np.complex64)
    A[40, 40] = 0.0
    dA = torch.as_tensor(A[None], device="cuda").contiguous()
    ipiv = torch.empty((1, n), dtype=torch.int32, device="cuda")
    info = torch.empty((1,), dtype=torch.int32, device="cuda")
    nat.call("ghost_bor_getrf", nat.F32, 1, n, nat.ptr(dA), n, n * n, nat.ptr(ipiv), nat.ptr(info), 0,
             nat.stream_handle())
    assert int(info.cpu()[0]) == 41


def test_bessel_rhs_against_scipy(pkg, torch):
    """Miller-recurrence Bessel tables inside the excitation kernel vs scipy jv,
    through rhs_mode at large orders and arguments."""
    from scipy import special as sp
    pts = pkg.bodies.sphere_generatrix(1.0, 30)
    k = 30.0
    f = k * 299_792_458.0 / (2 * math.pi)
    s = pkg.bor_solver.BorPecSolver(pts, f)
    g = s.g
    for m in (0, 7, 29, 40):
        for th in (0.0, 37.0, 90.0, 180.0):
            v = s.rhs_mode(m, th, "HH")
            t = math.radians(th)
            u = k * g.rho * math.sin(t)
            jm = lambda n: (1j) ** n * sp.jv(n, u)
            Ic = math.pi * (jm(m - 1) + jm(m + 1))
            Is = (math.pi / 1j) * (jm(m - 1) - jm(m + 1))
            P = np.exp(1j * k * math.cos(t) * g.z)
            want = np.concatenate([s.B_T @ (g.w * g.rho * P * g.trho * Is), s.B_T @ (g.w * g.rho * P * Ic)])
            assert rel(v, want) < 1e-12, (m, th)


@pytest.mark.parametrize("name", ["sphere_n24", "conesphere_n40"])
def test_near_band_double_float_matches_fp64(pkg, torch, name):
    """The double-float near projection (FP32 path) reproduces the FP64 near band."""
    D = load_golden(name)
    eng = pkg.engine
    nat = pkg._native
    prob = eng.BorGpuProblem(D["points"], float(D["freq_hz"]), D["thetas"], m_max=int(D["m_max"]))
    Mb = prob.m_max + 1
    b64 = torch.zeros((Mb, 4, prob.Nn, 5), dtype=torch.complex128, device="cuda")
    b32 = torch.zeros_like(b64)
    st = nat.stream_handle()
    prob.fill_near(prob.C, st, band=b64, precision=nat.F64)
    prob.fill_near(prob.C, st, band=b32, precision=nat.F32)
    torch.cuda.synchronize()
    prob.check_near_status()
    assert (b32 - b64).abs().max().item() < 1e-12 * b64.abs().max().item()


def test_residual_x32_presplit_matches(pkg, torch):
    """ghost_bor_residual_x32 on Z_far split in place into FP32 words gives the
    residual of the on-the-fly split bit for bit, and matches an FP64 residual."""
    nat = pkg._native
    rng = np.random.default_rng(5)
    Mb, Nn, nrhs = 3, 70, 33
    n = 2 * Nn
    Zh = (rng.standard_normal((Mb, n, n)) + 1j * rng.standard_normal((Mb, n, n)))
    Xh = (rng.standard_normal((Mb, n, nrhs)) + 1j * rng.standard_normal((Mb, n, nrhs))).astype(np.complex64)
    Bh = Zh @ Xh.astype(np.complex128) + 1e-3 * (rng.standard_normal((Mb, n, nrhs)) + 0j)
    Z = torch.as_tensor(Zh, device="cuda")
    X = torch.as_tensor(Xh, device="cuda")
    B = torch.as_tensor(Bh, device="cuda")
    masks = torch.full((Mb, 4), -1, dtype=torch.int32, device="cuda")
    out = []
    for split in (0, 1):
        R32 = torch.empty((Mb, n, nrhs), dtype=torch.complex64, device="cuda")
        R = torch.empty((Mb, n, nrhs), dtype=torch.complex128, device="cuda")
        norms = torch.empty((Mb, 2), dtype=torch.float64, device="cuda")
        if split:
            nat.call("ghost_bor_split_words", Mb, n, n, nat.ptr(Z), n, Z.stride(0), nat.stream_handle())
        nat.call("ghost_bor_residual_x32", Mb, n, nrhs, Nn, nat.ptr(Z), split, n, Z.stride(0), 0,
                 nat.ptr(masks), nat.ptr(X), nat.ptr(B), nrhs, B.stride(0), nat.ptr(R), nat.ptr(R32),
                 nat.ptr(norms), nat.stream_handle())
        torch.cuda.synchronize()
        out.append((R.cpu().numpy(), R32.cpu().numpy()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    ref = Bh - Zh @ Xh.astype(np.complex128)
    assert np.max(np.abs(out[1][0] - ref)) < 1e-6 * np.max(np.abs(Bh))


@pytest.mark.parametrize("Mb,Nn,nrhs", [(2, 70, 33), (3, 161, 97)])
def test_residual_exact_bf16_slices(pkg, torch, Mb, Nn, nrhs):
    """ghost_bor_residual_exact (Ozaki bf16 slices on tcgen05) against an FP64
    reference, with a near band and masked rows: far below the FP32-product
    floor of the split-word residual."""
    nat = pkg._native
    lib = nat.load()
    rng = np.random.default_rng(11)
    n = 2 * Nn
    Zh = rng.standard_normal((Mb, n, n)) + 1j * rng.standard_normal((Mb, n, n))
    Zh *= np.exp(rng.uniform(-3, 3, (Mb, n, 1)))            # rows of different magnitude
    Xh = (rng.standard_normal((Mb, n, nrhs)) + 1j * rng.standard_normal((Mb, n, nrhs))).astype(np.complex64)
    Xh *= np.exp(rng.uniform(-2, 2, (Mb, 1, nrhs))).astype(np.float32)
    band_h = rng.standard_normal((Mb, 4, Nn, 5)) + 1j * rng.standard_normal((Mb, 4, Nn, 5))
    Bh = Zh @ Xh.astype(np.complex128) * (1 + 1e-6 * rng.standard_normal((Mb, n, nrhs)))
    masks_h = np.full((Mb, 4), -1, dtype=np.int32)
    masks_h[:, 0] = 0
    masks_h[:, 1] = Nn
    # FP64 reference with the band (block (row half, col half) diagonals -2..2)
    ref = Bh - Zh @ Xh.astype(np.complex128)
    X64 = Xh.astype(np.complex128)
    for b in range(Mb):
        for half in range(2):
            for ch in range(2):
                for d in range(5):
                    for node in range(Nn):
                        jn = node + d - 2
                        if 0 <= jn < Nn:
                            ref[b, half * Nn + node] -= band_h[b, 2 * half + ch, node, d] * X64[b, ch * Nn + jn]
        ref[b, masks_h[b][masks_h[b] >= 0]] = 0
    Z = torch.as_tensor(Zh, device="cuda")
    X = torch.as_tensor(Xh, device="cuda")
    B = torch.as_tensor(Bh, device="cuda")
    band = torch.as_tensor(band_h, device="cuda")
    masks = torch.as_tensor(masks_h, device="cuda")
    R = torch.empty((Mb, n, nrhs), dtype=torch.complex128, device="cuda")
    R32 = torch.empty((Mb, n, nrhs), dtype=torch.complex64, device="cuda")
    norms = torch.empty((Mb, 2), dtype=torch.float64, device="cuda")
    nbytes = int(lib.ghost_bor_residual_exact_workspace(Mb, n, nrhs))
    work = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    nat.call("ghost_bor_residual_exact", Mb, n, nrhs, Nn, nat.ptr(Z), n, Z.stride(0), nat.ptr(band),
             nat.ptr(masks), nat.ptr(X), nat.ptr(B), nrhs, B.stride(0), nat.ptr(R), nat.ptr(R32),
             nat.ptr(norms), nat.ptr(work), nbytes, nat.stream_handle())
    torch.cuda.synchronize()
    assert int(work[:4].view(torch.int32)[0]) == 0
    got = R.cpu().numpy()
    scale = np.max(np.abs(Bh))
    assert np.max(np.abs(got - ref)) < 2e-9 * scale, np.max(np.abs(got - ref)) / scale
    nr = norms.cpu().numpy()           # accumulated in FP32 per thread (reported, not refined)
    np.testing.assert_allclose(nr[:, 0], np.sum(np.abs(got) ** 2, axis=(1, 2)), rtol=1e-5)
    np.testing.assert_allclose(nr[:, 1], np.sum(np.abs(Bh) ** 2, axis=(1, 2)), rtol=1e-5)


@pytest.mark.parametrize("m_max", [20, 50, 90, 200, 300])
def test_near_band_grouped_widths_match_fp64(pkg, torch, m_max):
    """The grouped double-float near kernel at 2, 4, 8 and 16 lanes per point
    pair (orders up to 32, 64, 128, 256) and the per-thread kernel beyond, against the
    FP64 near band, mode by mode.  A lane's step-G Chebyshev recurrence
    (at most 16 steps, multiplier 2 cos(G xi)) amplifies the double-float
    rounding by up to ~1/|sin(G xi)| per step: ~3e-12 (G = 8) to ~2e-11
    (G = 16) of the mode's largest entry, still ~1000x below the far fill's
    error."""
    eng = pkg.engine
    nat = pkg._native
    pts = pkg.bodies.cone_sphere_generatrix(0.5, 15.0, 60)
    prob = eng.BorGpuProblem(pts, 20.0 * 299792458.0 / (2 * math.pi), np.array([0.0, 90.0]), m_max=m_max)
    Mb = prob.m_max + 1
    b64 = torch.zeros((Mb, 4, prob.Nn, 5), dtype=torch.complex128, device="cuda")
    b32 = torch.zeros_like(b64)
    st = nat.stream_handle()
    prob.fill_near(prob.C, st, band=b64, precision=nat.F64)
    prob.fill_near(prob.C, st, band=b32, precision=nat.F32)
    torch.cuda.synchronize()
    prob.check_near_status()
    top = b64.abs().amax(dim=(1, 2, 3))
    err = (b32 - b64).abs().amax(dim=(1, 2, 3))
    print(f"\nM = {m_max}: max error / mode scale {float((err / top).max()):.2e}")
    assert torch.all(err <= 1e-10 * top), float((err / top).max())
