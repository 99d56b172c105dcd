"""The GPU dielectric (PMCHWT) solve's host orchestration against the
reference, on the CPU.

solve_bor_dielectric builds the 4 Nn system of every mode from fills that the
GPU tests pin one by one (EFIE far and near, the unit-weight impedance
brackets without mass term, the excitation, LU, far field).  Here each of
those fills is replaced by the oracle's block for the same call -- the same
semantics: add scale x the mode's block into the given (possibly strided)
block of the system -- and the LU / far-field entry points by their
mathematical definition, so the whole orchestration (interior medium as the
generatrix at f n, block placement and factors, the P column remap, the
masks, the right-hand-side columns, the two far-field halves, the m >= 0
symmetry and the mode truncation) runs on the CPU.  It must reproduce the
reference's own solve_bor_dielectric amplitudes for the lossless case of
tests/golden/pmchwt_sphere_n24.npz (eps_r = 4, mu_r = 1) to 1e-10.
"""
import math

import numpy as np
import pytest
import torch

import mock_device
from conftest import load_golden


@pytest.fixture
def emulated(monkeypatch, pkg, oracle):
    mock_device.install(monkeypatch, pkg)
    eng = pkg.engine
    pen = pkg.penetrable
    cache = {}

    def orc(prob):
        key = round(prob.freq_hz, 6)
        if key not in cache:
            o = oracle.OracleSolver(prob.gen.nodes, prob.freq_hz)
            o.prepare(prob.m_max, efie=True, workers=4, ibc_zs_pt=np.ones(o.geo.P))
            cache[key] = o
        return cache[key]

    media = []                       # (f in air, eps_r, mu_r) of the lossy media of a test

    def orc_ck(prob, k):
        for f, eps, mu in media:
            key = ("ck", round(f, 6), eps, mu)
            m_idx = complex(np.sqrt(complex(eps) * complex(mu)))
            m_idx = -m_idx if m_idx.imag > 0 else m_idx
            m_idx = -m_idx if m_idx.real < 0 else m_idx
            if abs(2 * math.pi * f / oracle.C0 * m_idx - k) <= 1e-9 * abs(k):
                if key not in cache:
                    o = oracle.OracleSolver(prob.gen.nodes, f, medium=(eps, mu))
                    o.prepare(prob.m_max, efie=True, workers=4, ibc_zs_pt=np.ones(o.geo.P))
                    cache[key] = o
                return cache[key]
        raise AssertionError(f"no medium registered for k = {k}")

    def blocks(prob, kind, o=None):
        o = orc(prob) if o is None else o
        M, Nn = prob.m_max, prob.Nn
        C = 1j * o.k * o.eta * 2.0 * math.pi
        out = []
        for m in range(M + 1):
            far = np.block([[b for b in o.efie_far_blocks(m)[:2]], [b for b in o.efie_far_blocks(m)[2:]]])
            if kind == "far":
                out.append(far)
            elif kind == "near":
                out.append(o.assemble_efie(m, M) / C - far)
            else:
                bf = [o.Bb[uv, m + M] for uv in range(4)]
                bt = o.rot_pv_blocks(m, M)
                if kind == "ibc_far":
                    out.append(np.block([[bf[0], bf[1]], [bf[2], bf[3]]]))
                else:
                    out.append(np.block([[bt[0] - bf[0], bt[1] - bf[1]], [bt[2] - bf[2], bt[3] - bf[3]]]))
        return torch.as_tensor(np.stack(out))

    def add(Z, scale, b):
        Z += complex(scale) * b

    monkeypatch.setattr(eng.BorGpuProblem, "fill_far",
                        lambda self, Z, prec, scale, st: add(Z, scale, blocks(self, "far")))
    monkeypatch.setattr(eng.BorGpuProblem, "fill_near",
                        lambda self, scale, st, band=None, Z=None, precision=None:
                        add(Z, scale, blocks(self, "near")))
    monkeypatch.setattr(eng.BorGpuProblem, "fill_far_ibc",
                        lambda self, Z, prec, scale, st: add(Z, scale, blocks(self, "ibc_far")))

    def near_ibc(self, scale, st, band=None, Z=None, mass=True):
        assert not mass
        add(Z, scale, blocks(self, "ibc_near"))
    monkeypatch.setattr(eng.BorGpuProblem, "fill_near_ibc", near_ibc)
    monkeypatch.setattr(eng.BorGpuProblem, "fill_far_ck",
                        lambda self, Z, k, scale, st: add(Z, scale, blocks(self, "far", orc_ck(self, k))))
    monkeypatch.setattr(eng.BorGpuProblem, "fill_near_ck",
                        lambda self, k, scale, st, Z=None, band=None:
                        add(Z, scale, blocks(self, "near", orc_ck(self, k))))
    monkeypatch.setattr(eng.BorGpuProblem, "fill_far_ibc_ck",
                        lambda self, Z, k, scale, st: add(Z, scale, blocks(self, "ibc_far", orc_ck(self, k))))

    def near_ibc_ck(self, k, scale, st, Z=None, band=None, mass=True):
        assert not mass
        add(Z, scale, blocks(self, "ibc_near", orc_ck(self, k)))
    monkeypatch.setattr(eng.BorGpuProblem, "fill_near_ibc_ck", near_ibc_ck)

    def excitation(self, B, coef_e, coef_h, st, h_weight=None):
        o = orc(self)
        for m in range(self.m_max + 1):
            for pol, c in (("VV", 0), ("HH", 1)):
                v = coef_e * o.rhs_efie(m, self.thetas, pol).T
                for r in self.masks[m]:
                    if r >= 0:
                        v[r] = 0.0
                B[m, :, c::2] = torch.as_tensor(v)
    monkeypatch.setattr(eng.BorGpuProblem, "excitation", excitation)

    def solve(Z, X, st):
        X.copy_(torch.linalg.solve(Z, X))
        return torch.zeros(X.shape[0], dtype=torch.int32)

    def residual(Z, X, B, st):
        R = Z @ X - B
        return torch.stack([(R.abs() ** 2).sum((1, 2)), (B.abs() ** 2).sum((1, 2))], dim=1)

    def farfield(prob, V, X, st):
        Nn = prob.Nn
        d = torch.ones(V.shape[1], dtype=torch.float64)
        d[Nn:] = -1.0
        sgn = torch.tensor([1.0 if c % 2 == 0 else -1.0 for c in range(X.shape[2])])
        pref = -1j * prob.k * 376.730313668 / (4.0 * math.pi)
        w = torch.as_tensor(np.where(np.arange(prob.m_max + 1) == 0, 1.0, 2.0))
        return pref * w[:, None] * sgn[None, :] * (d[None, :, None] * V * X).sum(1)

    monkeypatch.setattr(pen, "solve_fp64", solve)
    monkeypatch.setattr(pen, "residual_fp64", residual)
    monkeypatch.setattr(pen, "farfield_fp64", farfield)
    cache["media"] = media
    return cache


def test_dielectric_orchestration_matches_reference(pkg, emulated):
    D = load_golden("pmchwt_sphere_n24")
    assert tuple(D["media"][1]) == (4.0, 1.0)
    r = pkg.bor_solver.solve_bor_dielectric(D["points"], float(D["freq_hz"]), D["thetas"], 4.0, 1.0,
                                            n_modes=int(D["m_max"]), mode_tol=0.0)
    for pol in ("vv", "hh"):
        a, b = np.asarray(r[f"amp_{pol}"]), D[f"amp_{pol}_1"]
        assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b)), pol
    assert r["n_unknowns"] == 4 * len(D["points"]) and r["formulation"] == "pmchwt"
    assert r["linear_residual"] < 1e-12
    # the interior problem is the generatrix at f n
    assert sorted(k for k in emulated if k != "media") == sorted([round(float(D["freq_hz"]), 6),
                                                                  round(2.0 * float(D["freq_hz"]), 6)])


@pytest.mark.parametrize("case", [0, 2])
def test_lossy_dielectric_orchestration_matches_reference(pkg, emulated, case):
    """Lossy media (eps_r = 2.5 - 0.2j; eps_r = 2 - 0.1j with mu_r = 1.5 - 0.2j):
    the complex-wave-number fills of the interior, the rest as for a lossless
    body, against the reference's amplitudes."""
    D = load_golden("pmchwt_sphere_n24")
    eps, mu = (complex(x) for x in D["media"][case])
    f = float(D["freq_hz"])
    emulated["media"].append((f, eps, mu))
    r = pkg.bor_solver.solve_bor_dielectric(D["points"], f, D["thetas"], eps, mu,
                                            n_modes=int(D["m_max"]), mode_tol=0.0)
    for pol in ("vv", "hh"):
        a, b = np.asarray(r[f"amp_{pol}"]), D[f"amp_{pol}_{case}"]
        assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b)), pol


def test_medium_index_branch(pkg):
    """Index and impedance on the reference's causal branch (Im m <= 0, then
    Re m >= 0); a purely imaginary index (evanescent interior) is not taken."""
    pen = pkg.penetrable
    m, eta = pen.medium_index(4.0, 1.0)
    assert m == 2.0 and eta == pytest.approx(376.730313668 / 2.0, rel=1e-15)
    for eps, mu in ((2.5 - 0.2j, 1.0), (2.0, 1.5 - 0.2j), (-2.0 - 1j, 1.0), (-2.0, -1.0)):
        m, eta = pen.medium_index(eps, mu)
        assert m.imag <= 0.0 and m.real > 0.0
        assert abs(m * m - complex(eps) * complex(mu)) <= 1e-14 * abs(m * m)
        assert eta == pytest.approx(376.730313668 * complex(mu) / m, rel=1e-15)
    with pytest.raises(NotImplementedError, match="imaginary"):
        pen.medium_index(-2.0, 1.0)
    with pytest.raises(ValueError):
        pen.medium_index(float("nan"), 1.0)


def test_drop_in_medium_operators(pkg, oracle, emulated):
    """BorPecSolver(medium=(4, 1)): T with the medium's eta at f n and the
    remapped P equal the oracle's complex-medium operators; the exterior P
    equals the reference's."""
    D = load_golden("pmchwt_sphere_n24")
    M, f = int(D["m_max"]), float(D["freq_hz"])
    s = pkg.bor_solver.BorPecSolver(D["points"], f, medium=(4.0, 1.0))
    o = oracle.OracleSolver(D["points"], f, medium=(4.0, 1.0))
    o.prepare(M, efie=True, workers=4, ibc_zs_pt=np.ones(o.geo.P))
    for m in (0, 2, -3):
        T, P = s.assemble_mode(m, M), s.assemble_pmchwt_P(m, M)
        assert np.max(np.abs(T - o.assemble_efie(m, M))) <= 1e-12 * np.max(np.abs(T)), m
        assert np.max(np.abs(P - o.pmchwt_P(m, M))) <= 1e-12 * np.max(np.abs(P)), m
    se = pkg.bor_solver.BorPecSolver(D["points"], f)
    for m in D["modes"]:
        P = se.assemble_pmchwt_P(int(m), M)
        assert np.max(np.abs(P - D[f"Pe_{int(m)}"])) <= 1e-11 * np.max(np.abs(P)), m


def test_drop_in_lossy_medium_operators(pkg, oracle, emulated):
    """BorPecSolver(medium=(2.5 - 0.2j, 1)): T and P through the complex-k
    fills equal the reference's (tests/golden/pmchwt_sphere_n24.npz, modes 0
    and 2); its MFIE operator and streamed blocks are not provided."""
    D = load_golden("pmchwt_sphere_n24")
    M, f = int(D["m_max"]), float(D["freq_hz"])
    eps, mu = (complex(x) for x in D["media"][0])
    emulated["media"].append((f, eps, mu))
    s = pkg.bor_solver.BorPecSolver(D["points"], f, medium=(eps, mu))
    for m in D["modes"]:
        m = int(m)
        T, P = s.assemble_mode(m, M), s.assemble_pmchwt_P(m, M)
        assert np.max(np.abs(T - D[f"Ti_{m}"])) <= 1e-11 * np.max(np.abs(T)), m
        assert np.max(np.abs(P - D[f"Pi_{m}"])) <= 1e-11 * np.max(np.abs(P)), m
    with pytest.raises(NotImplementedError):
        s.assemble_mfie_mode(0, M)
    with pytest.raises(NotImplementedError):
        s.enable_streaming(M)
