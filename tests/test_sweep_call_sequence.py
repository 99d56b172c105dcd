"""The GPU sweep's host orchestration, run on the CPU.

Every C-ABI call a sweep makes (FP64 and FP32 + refinement; EFIE, CFIE, MFIE
and the surface-impedance EFIE) goes through a ctypes prototype of the
signature declared in _native.SIGNATURES -- the same argument conversion as
the real call -- and each formulation calls its own entry points.  Device
tensors are CPU tensors here and the entry points do nothing, so no number is
checked: the numerics are the GPU tests' business.
"""
import importlib

import numpy as np
import pytest
import torch

import mock_device
from conftest import load_golden

@pytest.fixture
def calls(monkeypatch, pkg):
    """CPU tensors for device memory, fake events and streams, and the entry
    points called (tests/mock_device.py)."""
    return mock_device.install(monkeypatch, pkg)


IBC_CALLS = {"ghost_bor_far_ibc", "ghost_bor_near_ibc", "ghost_bor_rhs_weighted"}


@pytest.mark.parametrize("precision", ["fp64", "fp32ir"])
@pytest.mark.parametrize("form,zs", [("efie", None), ("cfie", None), ("mfie", None),
                                     ("efie", "taper"), ("efie", 80 - 30j), ("mfie", 50.0)])
def test_sweep_calls_convert_to_declared_signatures(pkg, calls, precision, form, zs):
    D = load_golden("ibc_conesphere_n40")
    if isinstance(zs, str):
        zs = D["zs_taper"]
    prob = pkg.engine.BorGpuProblem(D["points"], float(D["freq_hz"]), D["thetas"][:5], m_max=4,
                                    formulation=form, zs=zs)
    res = prob.sweep(precision)
    assert res.dF.shape == (5, 2, 5)
    used = set(calls)
    fill = {"fp64": "ghost_bor_far_efie_masked", "fp32ir": "ghost_bor_far_efie_tc"}[precision]
    assert (fill in used) == (form != "mfie")
    assert ("ghost_bor_far_mfie" in used) == (form != "efie")
    # the impedance operator only with the EFIE part, its far-field vector always
    assert ({"ghost_bor_far_ibc", "ghost_bor_near_ibc"} <= used) == (zs is not None and form != "mfie")
    assert ("ghost_bor_rhs_weighted" in used) == (zs is not None)
    if zs is None:
        assert not used & IBC_CALLS
    assert "ghost_bor_farfield" in used


@pytest.mark.parametrize("precision", ["double", "auto"])
def test_solve_bor_with_impedance_and_monitor(pkg, calls, precision):
    """solve_bor(zs=...): a lossless Z_s on the closed cone-sphere switches the
    resonance monitor on (per-mode condition numbers, the reference's
    warning); a lossy one does not."""
    D = load_golden("ibc_conesphere_n40")
    bs = pkg.bor_solver
    r = bs.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"][:3], zs=-60j, n_modes=3,
                     mode_tol=0.0, table_precision=precision)
    assert "max_cond" in r and "median_cond" in r
    assert any("lossless" in w for w in r["warnings"])
    r = bs.solve_bor(D["points"], float(D["freq_hz"]), D["thetas"][:3], zs=D["zs_taper"], n_modes=3,
                     mode_tol=0.0, table_precision=precision)
    assert "max_cond" not in r and not any("lossless" in w for w in r["warnings"])
    assert IBC_CALLS <= set(calls)


def test_drop_in_impedance_operators(pkg, calls):
    """BorPecSolver.assemble_ibc_extra, farfield_mode(zs_pt) and the streamed
    IBC bracket blocks reach the impedance entry points; an all-zero Z_s needs
    no fill."""
    D = load_golden("ibc_conesphere_n40")
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]))
    zs = D["zs_taper"]
    Z = s.assemble_ibc_extra(-2, 4, zs[s.g.elem], zs)
    assert Z.shape == (2 * s.Nn, 2 * s.Nn)
    assert {"ghost_bor_far_ibc", "ghost_bor_near_ibc"} <= set(calls)
    del calls[:]
    assert not np.any(s.assemble_ibc_extra(1, 4, np.zeros(s.P), np.zeros(len(zs))))
    assert not calls
    s.farfield_mode(1, np.ones(2 * s.Nn, complex), 30.0, zs_pt=zs[s.g.elem])
    assert "ghost_bor_rhs_weighted" in calls
    for single in (False, True):
        s.enable_streaming(4, efie=False, ibc_zs_pt=zs[s.g.elem], single_blocks=single)
        assert len(s._stream.bracket_blocks("ibc", -3)) == 4
    with pytest.raises(ValueError):
        s._stream.bracket_blocks("mfie", 0)


def test_batched_sweep_and_adjoint_calls(pkg, calls):
    """The size-class batch (without graph capture) and the adjoint gradient
    make only declared calls too."""
    bodies = pkg.bodies
    bs = pkg.bor_solver
    items = [{"points": bodies.cone_sphere_generatrix(0.3, 15.0, n), "freq_hz": 1e9, "n_modes": 4}
             for n in (24, 30, 40)]
    out = bs.solve_bor_batch(items, [0.0, 45.0, 90.0], use_graphs=False, autotune=False)
    assert len(out) == 3 and all(len(r["amp_vv"]) == 3 for r in out)
    assert "ghost_bor_getrf" in calls
    del calls[:]
    adj = importlib.import_module("20260722_ghost_gb300.adjoint")
    r = torch.full((12,), 0.45, dtype=torch.float64, requires_grad=True)
    J = adj.bspline_rcs(r, 60, 1.5e9, np.arange(30.0, 40.01, 5.0), pol="HH", m_max=4)
    J.backward()
    assert r.grad is not None and r.grad.shape == (12,)
    assert "ghost_bor_far_efie_masked" in calls or "ghost_bor_far_efie_tc_masked" in calls


def test_dielectric_solve_calls(pkg, calls):
    """solve_bor_dielectric: the EFIE fills of both media into the diagonal
    blocks of the 4 Nn systems (row stride 4 Nn), the bracket fills without
    mass term, one excitation, the FP64 LU and two far-field calls."""
    D = load_golden("pmchwt_sphere_n24")
    r = pkg.bor_solver.solve_bor_dielectric(D["points"], float(D["freq_hz"]), D["thetas"][:3], 4.0, 1.0,
                                            n_modes=3, mode_tol=0.0)
    assert r["n_unknowns"] == 4 * len(D["points"])
    used = [c for c in calls if not c.endswith("_workspace")]
    assert used.count("ghost_bor_far_efie_masked") == 4 and used.count("ghost_bor_near_efie") == 4
    assert used.count("ghost_bor_far_ibc") == 2 and used.count("ghost_bor_near_ibc") == 2
    assert used.count("ghost_bor_farfield") == 2 and used.count("ghost_bor_rhs") == 1
    assert {"ghost_bor_getrf", "ghost_bor_getrs", "ghost_bor_residual64"} <= set(used)
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]), medium=(4.0, 1.0))
    assert s.assemble_mode(1, 3).shape == s.assemble_pmchwt_P(-1, 3).shape == (2 * s.Nn, 2 * s.Nn)


def test_lossy_dielectric_calls(pkg, calls):
    """A lossy medium's interior goes through the complex-wave-number fills."""
    D = load_golden("pmchwt_sphere_n24")
    pkg.bor_solver.solve_bor_dielectric(D["points"], float(D["freq_hz"]), D["thetas"][:2], 2.5 - 0.2j, 1.0,
                                        n_modes=3, mode_tol=0.0)
    used = [c for c in calls if not c.endswith("_workspace")]
    assert used.count("ghost_bor_far_efie_ck") == 2 and used.count("ghost_bor_near_efie_ck") == 2
    assert used.count("ghost_bor_far_ibc_ck") == 1 and used.count("ghost_bor_near_ibc_ck") == 1
    assert used.count("ghost_bor_far_efie_masked") == 2 and used.count("ghost_bor_far_ibc") == 1
    s = pkg.bor_solver.BorPecSolver(D["points"], float(D["freq_hz"]), medium=(2.5 - 0.2j, 1.0))
    del calls[:]
    assert s.assemble_mode(1, 3).shape == s.assemble_pmchwt_P(-1, 3).shape == (2 * s.Nn, 2 * s.Nn)
    assert {"ghost_bor_far_efie_ck", "ghost_bor_near_efie_ck", "ghost_bor_far_ibc_ck",
            "ghost_bor_near_ibc_ck"} <= set(calls)


def test_batch_with_impedance_bodies(pkg, calls):
    """solve_bor_batch with a per-body Z_s: the impedance bodies are swept one
    by one (their fills and far-field vector), the lossless-Z_s monitor as in
    solve_bor."""
    D = load_golden("ibc_conesphere_n40")
    items = [{"points": D["points"], "freq_hz": float(D["freq_hz"]), "n_modes": 3, "zs": D["zs_taper"]},
             {"points": D["points"], "freq_hz": float(D["freq_hz"]), "n_modes": 3, "zs": -40j}]
    out = pkg.bor_solver.solve_bor_batch(items, [0.0, 90.0])
    assert len(out) == 2
    assert "max_cond" not in out[0] and "max_cond" in out[1]
    assert any("lossless" in w for w in out[1]["warnings"])
    assert IBC_CALLS <= set(calls)
