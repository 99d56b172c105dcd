"""Adjoint RCS gradient on the GPU against central finite differences."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C0 = 299_792_458.0


def _case():
    radii = np.random.default_rng(0).uniform(0.3, 0.6, 12)
    k = 10.0
    return radii, 120, k * C0 / (2 * math.pi), np.arange(30.0, 60.0 + 1e-9, 2.5), 12


def test_adjoint_gradient_matches_central_differences(pkg):
    adj = pkg.adjoint
    radii, n_seg, f, th, M = _case()
    J, g = adj.bspline_rcs_and_gradient(radii, n_seg, f, th, pol="HH", m_max=M, precision="fp64")
    h = 1e-4
    for j in (1, 5, 10):
        rp, rm = radii.copy(), radii.copy()
        rp[j] += h
        rm[j] -= h
        Jp = adj.objective(adj._bspline_forward(rp, n_seg, f, th, "HH", M, "fp64", 1.0)[2], "HH")
        Jm = adj.objective(adj._bspline_forward(rm, n_seg, f, th, "HH", M, "fp64", 1.0)[2], "HH")
        fd = (Jp - Jm) / (2 * h)
        assert abs(g[j] - fd) < 1e-3 * max(abs(fd), 1e-3 * np.max(np.abs(g))), (j, g[j], fd)


def test_adjoint_fp32ir_matches_fp64_gradient(pkg):
    adj = pkg.adjoint
    radii, n_seg, f, th, M = _case()
    J64, g64 = adj.bspline_rcs_and_gradient(radii, n_seg, f, th, pol="HH", m_max=M, precision="fp64")
    J32, g32 = adj.bspline_rcs_and_gradient(radii, n_seg, f, th, pol="HH", m_max=M, precision="fp32ir")
    assert abs(J32 - J64) < 1e-4 * abs(J64)
    assert np.max(np.abs(g32 - g64)) < 1e-3 * np.max(np.abs(g64))


def test_autograd_function(pkg):
    import torch
    adj = pkg.adjoint
    radii, n_seg, f, th, M = _case()
    r = torch.tensor(radii, dtype=torch.float64, requires_grad=True)
    J = adj.bspline_rcs(r, n_seg, f, th, pol="HH", m_max=M, precision="fp64")
    J.backward()
    J_ref, g_ref = adj.bspline_rcs_and_gradient(radii, n_seg, f, th, pol="HH", m_max=M, precision="fp64")
    assert abs(J.item() - J_ref) < 1e-10 * abs(J_ref)
    assert np.max(np.abs(r.grad.numpy() - g_ref)) < 1e-8 * np.max(np.abs(g_ref))


@pytest.mark.parametrize("precision", ["fp64", "fp32ir"])
def test_adjoint_matches_reference_finite_differences(pkg, precision):
    """Against the reference's own FP64 solve_bor: central differences of the
    mean HH cross-section for every radius at h = 1e-4 and 5e-5 m
    (tests/golden/bspline_fd_ref.npz, made by tests/golden/make_fullsize_golden.py),
    Richardson-extrapolated; the objective itself to 1e-10."""
    from conftest import load_golden
    D = load_golden("bspline_fd_ref")
    adj = pkg.adjoint
    radii, n_seg, f, th, M = _case()
    np.testing.assert_array_equal(radii, D["radii"])
    np.testing.assert_array_equal(th, D["thetas"])
    J, g = adj.bspline_rcs_and_gradient(radii, n_seg, f, th, pol="HH", m_max=M, precision=precision)
    g1 = (D["Jp_h1"] - D["Jm_h1"]) / (2 * D["h1"])
    g2 = (D["Jp_h2"] - D["Jm_h2"]) / (2 * D["h2"])
    fd = (4.0 * g2 - g1) / 3.0
    assert abs(J - float(D["J0"])) < (1e-10 if precision == "fp64" else 1e-6) * abs(float(D["J0"]))
    assert np.max(np.abs(g - fd)) < 1e-3 * np.max(np.abs(fd)), (g, fd)
