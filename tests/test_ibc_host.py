"""The surface-impedance (IBC-EFIE) fill, checked on the host.

The GPU IBC fills are the IBC instantiations of the MFIE bracket kernels
(csrc/mfie_fill.cu): another per-pair coefficient set, the opposite sign of
the bracket term and a complex Z_s per source element.  The coefficient and
entry code they compile (csrc/brackets.cuh) is built here for the host with
g++ (tests/brackets_host.cpp) and replayed against the oracle, which is
pinned to the reference's IBC operator (tests/test_oracle_ibc.py):

* both coefficient sets reproduce the oracle's bracket samples on far and
  near point pairs;
* the far fill's formulation with the IBC set, the per-element Z_s weights
  and the entry rule reproduces the oracle's Z_s-weighted far IBC blocks;
* the entry rule is -s K + s M/2 for the MFIE and s Z_s (K + M/2) for the IBC;
* the per-element mass contributions weighted by Z_s give the oracle's
  Z_s mass term;
* the device IBC sampler's loop body (ghost_bor_sample_ibc) equals the
  reference's own compiled sample_ibc and the oracle's brackets.

Plus the host side of solve_bor(zs=...): Z_s parsing and its errors, before
any device work.
"""
import ctypes
import importlib
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import load_golden

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "20260722_ghost_gb300", "csrc")


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ is not available")
    out = str(tmp_path_factory.mktemp("brackets") / "libbrackets_host.so")
    subprocess.run([gxx, "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{CSRC}",
                    os.path.join(HERE, "brackets_host.cpp"), "-o", out], check=True)
    lib = ctypes.CDLL(out)
    dp = ctypes.POINTER(ctypes.c_double)
    for name in ("host_bracket_coefs", "host_bracket_entry"):
        getattr(lib, name).argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        getattr(lib, name).restype = None
    lib.host_sample_ibc.argtypes = SAMPLER_ARGS
    lib.host_sample_ibc.restype = None
    lib.host_complex_k.argtypes = [ctypes.c_int, dp, dp]
    lib.host_complex_k.restype = None
    return lib


_dp = ctypes.POINTER(ctypes.c_double)
SAMPLER_ARGS = [ctypes.c_int] * 3 + [_dp] * 8 + [ctypes.c_double, _dp, _dp] + [_dp] * 4


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def coefs(shim, ibc, rp, zp, trp, tzp, rq, zq, trq, tzq):
    """c0..c5 of every pair (broadcast inputs), from the compiled kernel code."""
    arrs = np.broadcast_arrays(rp, zp, trp, tzp, rq, zq, trq, tzq)
    shape = arrs[0].shape
    pairs = np.ascontiguousarray(np.stack([a.ravel() for a in arrs], axis=1), dtype=np.float64)
    out = np.empty((pairs.shape[0], 6))
    shim.host_bracket_coefs(int(ibc), pairs.shape[0], _ptr(pairs), _ptr(out))
    return [out[:, i].reshape(shape) for i in range(6)]


@pytest.mark.parametrize("kind", ["mfie", "ibc"])
def test_bracket_coefficients_reproduce_oracle_samples(oracle, shim, kind):
    """p (c0 + c1 s2), p sin(xi) c4, p sin(xi) c5, p (c2 + c3 s2) = the oracle's
    tt, tf, ft, ff bracket samples, far pairs and pairs a few 1e-3 apart."""
    rng = np.random.default_rng(11)
    n = 400
    rp, rq = rng.uniform(0.05, 1.0, n), rng.uniform(0.05, 1.0, n)
    zp, zq = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    a, b = rng.uniform(0, 2 * math.pi, n), rng.uniform(0, 2 * math.pi, n)
    trp, tzp, trq, tzq = np.cos(a), np.sin(a), np.cos(b), np.sin(b)
    rq[:100] = rp[:100] + rng.uniform(-3e-3, 3e-3, 100)
    zq[:100] = zp[:100] + rng.uniform(-3e-3, 3e-3, 100)
    xi = rng.uniform(-math.pi, math.pi, (n, 64))
    xi[:100, :8] = rng.uniform(-1e-2, 1e-2, (100, 8))
    k = 30.0
    grid = oracle._ibc_bracket_grid if kind == "ibc" else oracle._mfie_bracket_grid
    want = grid(rp, zp, trp, tzp, rq, zq, trq, tzq, k, xi)
    c = [x[:, None] for x in coefs(shim, kind == "ibc", rp, zp, trp, tzp, rq, zq, trq, tzq)]
    dr, dz = (rp - rq)[:, None], (zp - zq)[:, None]
    R = np.sqrt(dr ** 2 + dz ** 2 + 4 * (rp * rq)[:, None] * np.sin(xi / 2) ** 2)
    p = (1 + 1j * k * R) * np.exp(-1j * k * R) / (4 * np.pi * R ** 3)
    s2, sx = np.sin(xi / 2) ** 2, np.sin(xi)
    got = (p * (c[0] + c[1] * s2), p * sx * c[4], p * sx * c[5], p * (c[2] + c[3] * s2))
    scale = np.abs(p) * (1.0 + np.abs(dz) + rp[:, None] + rq[:, None])
    for g_, w_ in zip(got, want):
        assert np.max(np.abs(g_ - w_) / scale) < 1e-13


def _run_sampler(fn):
    rng = np.random.default_rng(2)
    nr, npp, nx = 5, 9, 32
    a = [np.ascontiguousarray(rng.uniform(0.01, 1, nr)) for _ in range(4)]
    b = [np.ascontiguousarray(rng.uniform(0.01, 1, npp)) for _ in range(4)]
    xi = 2 * np.pi * np.arange(nx) / nx - np.pi
    cx, sx = np.ascontiguousarray(np.cos(xi)), np.ascontiguousarray(np.sin(xi))
    outs = [np.empty((nr, npp, nx), np.complex128) for _ in range(4)]
    fn(nr, npp, nx, *[_ptr(v) for v in a], *[_ptr(v) for v in b], 7.5, _ptr(cx), _ptr(sx),
       *[_ptr(o) for o in outs])
    return a, b, xi, outs


def test_ibc_sampler_matches_reference_and_oracle(oracle, shim):
    """The device IBC sampler's loop body (ghost_bor_sample_ibc, factors from
    csrc/brackets.cuh) run on the host: equal to the reference's own compiled
    sample_ibc (oracle/_ref, when the reference tree was available to build it)
    to rounding, and to the oracle's NumPy brackets."""
    a, b, xi, outs = _run_sampler(shim.host_sample_ibc)
    nr, npp, nx = outs[0].shape
    one = np.ones((nr, npp))
    F = oracle._ibc_bracket_grid(*[(v[:, None] * one).ravel() for v in a],
                                 *[(v[None, :] * one).ravel() for v in b], 7.5,
                                 np.broadcast_to(xi, (nr * npp, nx)))
    for o, f in zip(outs, F):
        f = f.reshape(nr, npp, nx)
        assert np.max(np.abs(o - f)) <= 1e-13 * np.max(np.abs(f))
    ref_path = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "bor_stream_kernel.so")
    if not os.path.exists(ref_path):
        pytest.skip("reference sampler not built (reference tree absent)")
    ref = ctypes.CDLL(ref_path)
    ref.sample_ibc.argtypes = SAMPLER_ARGS
    ref.sample_ibc.restype = None
    _, _, _, routs = _run_sampler(ref.sample_ibc)
    for o, r in zip(outs, routs):
        assert np.max(np.abs(o - r)) <= 1e-15 * np.max(np.abs(r))


def test_bracket_entry_rule(shim):
    rng = np.random.default_rng(5)
    n = 64
    v = rng.standard_normal((n, 5))
    K = v[:, 0] + 1j * v[:, 1]
    s = v[:, 3] + 1j * v[:, 4]
    for ibc, want in ((0, s * (-K + v[:, 2])), (1, s * (K + v[:, 2]))):
        out = np.empty((n, 2))
        inp = np.ascontiguousarray(v)
        shim.host_bracket_entry(ibc, n, _ptr(inp), _ptr(out))
        assert np.max(np.abs(out[:, 0] + 1j * out[:, 1] - want)) <= 1e-15 * np.max(np.abs(want))


def test_far_ibc_fill_with_impedance_weights(oracle, pkg, shim):
    """The far IBC fill's formulation emulated on the host: half-grid
    transforms C[p], C[p s2], S of p with the kernel's tables, the compiled
    IBC coefficients, the -j sine convention, the T w rho Galerkin weights, and
    the entry rule with s = Z_s of the source element -- equals the oracle's
    far IBC blocks with Z_s in the source weights (a tapered complex Z_s with
    a bare nose), m = 0..M."""
    geom = pkg.geometry
    pts = pkg.bodies.cone_sphere_generatrix(0.3, 15.0, 24)
    k, M = 20.0, 6
    o = oracle.OracleSolver(pts, k * oracle.C0 / (2 * math.pi))
    N = o.geo.ne
    t = (np.arange(N) + 0.5) / N
    zs = (60.0 + 240.0 * t) - 1j * (30.0 + 20.0 * np.cos(3.0 * t))
    zs[:4] = 0.0
    o.build_far(M, efie=False, ibc_zs_pt=zs[o.geo.elem])
    gen = geom.Generatrix(pts)
    geo = geom.pack_geo(geom.gauss_on_generatrix(gen, 4))
    P = 4 * N
    tab, s2 = geom.bracket_tables(geom.n_xi_bracket(k, float(np.max(gen.nodes[:, 0])), M), M)
    rho, z, tr, tz = geo[0], geo[1], geo[9], geo[10]
    e_of = np.arange(P) // 4
    pi, qi = np.meshgrid(np.arange(P), np.arange(P), indexing="ij")
    far = (np.abs(e_of[pi] - e_of[qi]) >= 2)[..., None]
    R = np.maximum(np.sqrt(((rho[pi] - rho[qi]) ** 2 + (z[pi] - z[qi]) ** 2)[..., None]
                           + (4 * rho[pi] * rho[qi])[..., None] * s2), 1e-30)
    p = (1 + 1j * k * R) * np.exp(-1j * k * R) / R ** 3
    T = np.einsum("pqj,tjm->tpqm", p, tab)
    c = [x[..., None] for x in coefs(shim, True, rho[pi], z[pi], tr[pi], tz[pi], rho[qi], z[qi],
                                     tr[qi], tz[qi])]
    K = [c[0] * T[0] + c[1] * T[1], -1j * c[4] * T[2], -1j * c[5] * T[2], c[2] * T[0] + c[3] * T[1]]
    W = np.zeros((N + 1, P))
    W[e_of, np.arange(P)] += geo[3]
    W[e_of + 1, np.arange(P)] += geo[4]
    wsrc = zs[e_of][None, :, None]                # Z_s of the source element, per source point
    scale = np.max(np.abs(o.Bb))
    for uv in range(4):
        got = np.einsum("ip,pqm,jq->mij", W, K[uv] * far * wsrc, W)
        assert np.max(np.abs(got - o.Bb[uv, M:])) <= 1e-13 * scale, uv


def test_impedance_mass_from_element_contributions(pkg, oracle):
    """Sum over elements of Z_s(e) x the element mass contributions (the self
    pairs of the near IBC fill) = the oracle's Z_s-weighted mass term."""
    geom = pkg.geometry
    D = load_golden("ibc_conesphere_n40")
    o = oracle.OracleSolver(D["points"], float(D["freq_hz"]))
    gen = geom.Generatrix(D["points"])
    g = geom.gauss_on_generatrix(gen, 4)
    N = gen.n_elems
    em = geom.element_mass(g, N)
    zs = D["zs_taper"]
    got = np.zeros((N + 1, N + 1), dtype=complex)
    for e in range(N):
        for ab in range(4):
            got[e + ab // 2, e + ab % 2] += zs[e] * em[e, ab]
    want = o.mass(zs[o.geo.elem])
    assert np.max(np.abs(got - want)) <= 1e-14 * np.max(np.abs(want))


def test_impedance_parsing_and_errors(pkg):
    """Z_s as solve_bor reads it (bor_solver.py:848-866): scalar -> every
    element, per-element array checked for length, all zero -> PEC; CFIE with
    a non-zero Z_s and a wrong length are ValueErrors raised before any device
    work (so also without a GPU)."""
    eng = pkg.engine
    assert eng.impedance_per_element(None, 5) is None
    assert eng.impedance_per_element(0.0, 5) is None
    assert eng.impedance_per_element(np.zeros(5), 5) is None
    np.testing.assert_array_equal(eng.impedance_per_element(50 - 2j, 3), np.full(3, 50 - 2j))
    v = np.array([0, 1 + 1j, 2])
    np.testing.assert_array_equal(eng.impedance_per_element(v, 3), v.astype(complex))
    with pytest.raises(ValueError):
        eng.impedance_per_element(np.ones(4), 3)
    with pytest.raises(ValueError):
        eng.impedance_per_element(np.array([1.0, np.nan, 2.0]), 3)
    bs = importlib.import_module("20260722_ghost_gb300.bor_solver")
    pts = pkg.bodies.sphere_generatrix(1.0, 12)
    with pytest.raises(ValueError, match="CFIE with surface impedance"):
        bs.solve_bor(pts, 3e8, [0.0], formulation="cfie", zs=50.0)
    with pytest.raises(ValueError, match="one entry per generatrix element"):
        bs.solve_bor(pts, 3e8, [0.0], zs=np.ones(5))
    s = bs.BorPecSolver(pts, 3e8)
    with pytest.raises(NotImplementedError):
        s._zs_elem(np.arange(s.P, dtype=complex))          # not constant on each element
    ze = np.arange(12, dtype=complex)
    np.testing.assert_array_equal(s._zs_elem(ze[s.g.elem], ze), ze)


def test_complex_wave_number_samples(shim):
    """The lossy-medium fills' samples (csrc/medium.cuh, compiled for the
    host): e^{-jkR}/R, (1 + jkR) e^{-jkR}/R^3 and 1/k^2 for k = k_r + j k_i,
    k_i <= 0, equal the complex formulas."""
    rng = np.random.default_rng(8)
    n = 500
    v = np.ascontiguousarray(np.stack([rng.uniform(1e-3, 3.0, n), rng.uniform(0.5, 200.0, n),
                                       -rng.uniform(0.0, 30.0, n)], axis=1))
    out = np.empty((n, 6))
    shim.host_complex_k(n, _ptr(v), _ptr(out))
    R, k = v[:, 0], v[:, 1] + 1j * v[:, 2]
    for got, want in ((out[:, 0] + 1j * out[:, 1], np.exp(-1j * k * R) / R),
                      (out[:, 2] + 1j * out[:, 3], (1 + 1j * k * R) * np.exp(-1j * k * R) / R ** 3),
                      (out[:, 4] + 1j * out[:, 5], 1.0 / k ** 2)):
        assert np.max(np.abs(got - want) / np.abs(want)) < 1e-13
