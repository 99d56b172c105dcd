"""The GPU sweep's host orchestration, run on the CPU.

Every C-ABI call a sweep makes (FP64 and FP32 + refinement; EFIE, CFIE, MFIE
and the surface-impedance EFIE) goes through a ctypes prototype of the
signature declared in _native.SIGNATURES -- the same argument conversion as
the real call -- and each formulation calls its own entry points.  Device
tensors are CPU tensors here and the entry points do nothing, so no number is
checked: the numerics are the GPU tests' business.
"""
import ctypes
import importlib

import numpy as np
import pytest
import torch

from conftest import load_golden

_REAL_DEVICE = torch.device


def _cpu(d):
    return "cpu" if d is not None and str(d).startswith("cuda") else d


class _Event:
    def __init__(self, *a, **k):
        pass

    def record(self, *a, **k):
        pass

    def elapsed_time(self, other):
        return 1.0


class _Stream:
    cuda_stream = 0


@pytest.fixture
def calls(monkeypatch, pkg):
    """Route torch's CUDA allocations to zero-filled CPU tensors, fake the
    CUDA events and streams, and record the entry points called."""
    zero_for = {"empty": torch.zeros, "empty_like": torch.zeros_like}
    for name in ("zeros", "ones", "as_tensor", "tensor", "full", "arange", "zeros_like", "empty",
                 "empty_like"):
        fn = zero_for.get(name, getattr(torch, name))

        def wrapped(*a, _fn=fn, **k):
            if "device" in k:
                k["device"] = _cpu(k["device"])
            return _fn(*a, **k)
        monkeypatch.setattr(torch, name, wrapped)
    to = torch.Tensor.to

    def tensor_to(self, *a, **k):
        a = tuple(_cpu(x) if isinstance(x, (str, _REAL_DEVICE)) else x for x in a)
        if "device" in k:
            k["device"] = _cpu(k["device"])
        return to(self, *a, **k)
    monkeypatch.setattr(torch.Tensor, "to", tensor_to)
    for name, val in (("is_available", lambda: True), ("mem_get_info", lambda *a: (1 << 40, 1 << 40)),
                      ("memory_reserved", lambda *a: 0), ("memory_allocated", lambda *a: 0),
                      ("Event", _Event), ("synchronize", lambda *a: None),
                      ("current_stream", lambda *a: _Stream())):
        monkeypatch.setattr(torch.cuda, name, val)

    nat, eng = pkg._native, pkg.engine

    class TorchOnCpu:
        def __getattr__(self, n):
            return getattr(torch, n)

        def device(self, d=None, *a):
            return _REAL_DEVICE(_cpu(d) if d is not None else "cpu", *a)

    monkeypatch.setattr(eng, "_torch", lambda: TorchOnCpu())
    log = []
    protos = {}
    for name, (res, args) in nat.SIGNATURES.items():
        if res in (ctypes.c_int, ctypes.c_longlong):
            ret = (1 << 20) if res is ctypes.c_longlong else 0
            protos[name] = ctypes.CFUNCTYPE(res, *args)(lambda *a, _r=ret: _r)

    class Lib:
        def __getattr__(self, name):
            fn = protos[name]

            def g(*a):
                log.append(name)
                return fn(*a)
            return g

    def call(name, *args):
        res, argt = nat.SIGNATURES[name]
        assert len(args) == len(argt), (name, len(args), len(argt))
        log.append(name)
        return protos[name](*args)

    monkeypatch.setattr(nat, "load", lambda *a, **k: Lib())
    monkeypatch.setattr(nat, "call", call)
    return log


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
