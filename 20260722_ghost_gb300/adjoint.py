"""Adjoint gradient of the monostatic RCS with respect to generatrix shape
parameters, on the GPU, behind a torch.autograd.Function.

For one mode m and one aspect angle the monostatic far field is, by
reciprocity (the farfield kernel of this package),

    F = s c (D V)^T x,    Z x = V,    c = -j k eta0 / (4 pi),

s = +1 for VV (F_theta), -1 for HH (F_phi), D = diag(I, -I), so

    dF = s c [ (D x)^T dV + y^T dV - y^T dZ x ],    Z^T y = D V.

The Galerkin BoR EFIE operator satisfies Z^T = D Z D up to the symmetry of
its quadrature (~1e-5 relative: the near cells use a source order one above
the test order), so y = D x + delta with Z^T delta = s := D V - Z^T D x, a
small right-hand side; delta = D Z^-1 D s to first order in the asymmetry,
one solve with the factors of the sweep.  s uses the unfactored fl32(Z)
(its error, 6e-8, is far below the asymmetry it resolves).

For J = mean over angles of sigma = 4 pi |F|^2 (F summed over m with the mode
weights 1, 2, 2, ...), dJ/dp = mean 8 pi Re(conj(F) dF/dp).

dZ/dp and dV/dp are recomputed in the backward pass (nothing of size n^2 is
stored per parameter): for parameter p the generatrix nodes move by
+-h dnodes/dp, and the operator change is filled by the GPU kernels directly
into one buffer as (Z(+h) - Z(-h)) / 2h, restricted to the element pairs that
touch a moved element (far pairs: ghost_bor_far_efie_tc_masked for FP32+IR
sweeps, ghost_bor_far_efie_masked in FP64 for FP64 sweeps; near pairs: a
subset of the near-pair table through the double-float or the FP64 near
kernel); dV likewise from two FP64 excitation launches.  The quadrature orders (n_xi, near tail orders) stay those of the
unperturbed body, so the derivative is that of the discrete operator.

Shape parameters of the benchmark body (bodies.bspline_body): the control radii
of a clamped cubic B-spline radius profile whose nodes sit at fixed spline
parameters, so d rho_i / d r_j = B_ij and z does not move.
"""

from __future__ import annotations

import math
from typing import Optional, Sequence

import numpy as np

from . import _native as nat
from .bodies import bspline_body
from .engine import BorGpuProblem
from .geometry import ETA0, Generatrix, gauss_on_generatrix, pack_geo

_POLS = {"VV": 0, "THETA": 0, "TM": 0, "HH": 1, "PHI": 1, "TE": 1}


class _Tables:
    """Device geometry tables of a (perturbed) generatrix."""

    def __init__(self, torch, device, points):
        gen = Generatrix(np.asarray(points, float))
        g = gauss_on_generatrix(gen, 4)
        f64 = torch.float64
        elem = np.stack([gen.lengths, gen.trho, gen.tz])
        self.geo = torch.as_tensor(pack_geo(g), dtype=f64, device=device)
        self.nodes = torch.as_tensor(np.ascontiguousarray(gen.nodes), dtype=f64, device=device)
        self.elem = torch.as_tensor(np.ascontiguousarray(elem), dtype=f64, device=device)


class ShapeGradient:
    """dJ/dp for J = mean_theta sigma_pol(theta) of one body, given the
    converged solution of its sweep (EFIE, PEC)."""

    def __init__(self, prob: BorGpuProblem, res, F: np.ndarray, pol: str, h: float = 1e-5):
        if prob.alpha != 1.0:
            raise NotImplementedError("the adjoint gradient covers the EFIE formulation")
        self.prob = prob
        self.torch = prob.torch
        # FP32+IR sweeps take the operator change from the fills of that path
        # (tensor-core far transform, double-float near kernel): their errors,
        # ~4e-9 and ~3e-11 of |Z|, are ~1e-6 of a dZ that varies on the element
        # scale; FP64 sweeps keep the FP64 fills
        self.fast = res.lu["prec"] == nat.F32 and prob.far_tc
        self.pol = _POLS[pol.upper()]
        self.F = F                               # [2, T] complex128, host
        self.h = float(h)
        t = self.torch
        Mb, n, T = prob.m_max + 1, prob.n, prob.T
        self.cols = t.arange(T, device=prob.device) * 2 + self.pol
        d = t.ones(n, dtype=t.float64, device=prob.device)
        d[prob.Nn:] = -1.0
        self.Xp = res.X[:, :, self.cols].contiguous()          # [Mb, n, T]
        self.DX = (d[None, :, None] * self.Xp).contiguous()
        self.Y = self._adjoint(res, d)
        self.Xp32 = self.Xp.to(t.complex64)
        self.mode_w = prob.d_mode_w.to(t.complex128)
        self.dZ = t.empty((Mb, n, n), dtype=t.complex128, device=prob.device)
        self.V2 = t.empty((2, Mb, n, prob.nrhs), dtype=t.complex128, device=prob.device)
        self.rhs_work = None

    def _adjoint(self, res, d):
        """y = Z^-T D V = D x + D Z^-1 D s, s = D V - Z^T D x (see the module docstring)."""
        t = self.torch
        p = self.prob
        lu = res.lu
        Mb, n, T = p.m_max + 1, p.n, p.T
        V = res.Ve[:, :, self.cols]
        DV = d[None, :, None] * V
        op = lu["op"]
        ZtDx = t.bmm(op.transpose(1, 2), self.DX.to(op.dtype)).to(t.complex128)
        Ds = d[None, :, None] * (DV - ZtDx)
        rdt = t.complex64 if lu["prec"] == nat.F32 else t.complex128
        w = Ds.to(rdt).contiguous()
        nat.call("ghost_bor_getrs", lu["prec"], Mb, n, T, nat.ptr(lu["A"]), n, lu["A"].stride(0),
                 nat.ptr(lu["ipiv"]), nat.ptr(w), T, w.stride(0), nat.ptr(lu["work"]), nat.stream_handle())
        return (self.DX + d[None, :, None] * w.to(t.complex128)).contiguous()

    def _fill(self, tabs: _Tables, scale: complex, emask, pairs, tails, st):
        p = self.prob
        n = p.n
        if self.fast:
            ws = p._far_tc_work(st)
            nat.call("ghost_bor_far_efie_tc_masked", p.N, p.m_max, p.n_xi, p.k, scale.real, scale.imag,
                     nat.ptr(tabs.geo), nat.ptr(emask), nat.ptr(ws), ws.numel(), nat.ptr(self.dZ), n,
                     self.dZ.stride(0), st)
        else:
            nat.call("ghost_bor_far_efie_masked", nat.F64, p.N, p.m_max, p.n_xi, p.k, scale.real, scale.imag,
                     nat.ptr(tabs.geo), nat.ptr(p.d_dct), nat.ptr(p.d_sin2), nat.ptr(self.dZ), n,
                     self.dZ.stride(0), nat.ptr(emask), 0, st)
        if pairs is not None:
            work, nbytes = p._near_work("ghost_bor_near_workspace")
            nat.call("ghost_bor_near_efie", nat.F32 if self.fast else nat.F64, p.N, p.m_max, p.k,
                     scale.real, scale.imag,
                     nat.ptr(tabs.nodes), nat.ptr(tabs.elem), int(pairs.shape[0]), nat.ptr(pairs),
                     nat.ptr(tails), nat.ptr(p.d_cells), p.near.cells.shape[1], nat.ptr(p.d_core),
                     nat.ptr(p.d_tail), p.near.tail_gl.shape[1], 0, nat.ptr(self.dZ), n, self.dZ.stride(0),
                     p.n_tail_max, nat.ptr(work), nbytes, st)

    def _excite(self, tabs: _Tables, out, st):
        p = self.prob
        lib = nat.load()
        if self.rhs_work is None:
            nbytes = int(lib.ghost_bor_rhs_workspace(p.N, p.m_max, p.T))
            self.rhs_work = self.torch.empty(nbytes, dtype=self.torch.uint8, device=p.device)
        nat.call("ghost_bor_rhs", p.N, p.m_max, p.T, p.k, 1.0, 0.0, nat.ptr(tabs.geo), nat.ptr(p.d_thetas),
                 nat.ptr(p.d_masks), nat.ptr(out), out.shape[-1], out.stride(0), nat.ptr(self.rhs_work), st)

    def directional(self, dnodes: np.ndarray) -> float:
        """dJ along a node displacement field dnodes [Nn, 2] (rho, z)."""
        t = self.torch
        p = self.prob
        st = nat.stream_handle()
        h = self.h
        base = p.gen.nodes
        moved = np.any(dnodes != 0.0, axis=1)
        emask_h = (moved[:-1] | moved[1:]).astype(np.uint8)
        if not emask_h.any():
            return 0.0
        emask = t.as_tensor(emask_h, device=p.device)
        sel = np.flatnonzero(emask_h[p.near.pairs[:, 0]] | emask_h[p.near.pairs[:, 1]])
        pairs = t.as_tensor(np.ascontiguousarray(p.near.pairs[sel]), dtype=t.int32, device=p.device)
        tails = t.as_tensor(np.ascontiguousarray(p.near.tails[sel]), dtype=t.int32, device=p.device)
        plus = _Tables(t, p.device, base + h * dnodes)
        minus = _Tables(t, p.device, base - h * dnodes)
        # dZ = (Z(+h) - Z(-h)) / 2h on the pairs that move, dV likewise
        self.dZ.zero_()
        sc = p.C / (2.0 * h)
        self._fill(plus, sc, emask, pairs, tails, st)
        self._fill(minus, -sc, emask, pairs, tails, st)
        self._excite(plus, self.V2[0], st)
        self._excite(minus, self.V2[1], st)
        dV = (self.V2[0][:, :, self.cols] - self.V2[1][:, :, self.cols]) / (2.0 * h)
        # dZ x in complex64: the central difference is accurate to ~1e-9 only
        dZx = t.bmm(self.dZ.to(t.complex64), self.Xp32).to(t.complex128)
        g = t.sum(self.DX * dV + self.Y * (dV - dZx), dim=1)       # [Mb, T]
        c = -1j * p.k * ETA0 / (4.0 * math.pi)
        s = 1.0 if self.pol == 0 else -1.0
        dF = s * c * t.sum(self.mode_w[:, None] * g, dim=0)          # [T]
        Fp = t.as_tensor(self.F[self.pol], device=p.device)
        dJ = t.mean(8.0 * math.pi * (Fp.conj() * dF).real)
        self._keep = (plus, minus, emask, pairs, tails)               # outlive the launches
        return float(dJ)


def objective(F: np.ndarray, pol: str) -> float:
    """mean over angles of sigma_pol = 4 pi |F_pol|^2 (linear m^2)."""
    return float(np.mean(4.0 * math.pi * np.abs(F[_POLS[pol.upper()]]) ** 2))


def _bspline_forward(radii, n_seg, freq_hz, thetas_deg, pol, m_max, precision, half_length):
    pts, Bsp = bspline_body(radii, n_seg, half_length)
    prob = BorGpuProblem(pts, freq_hz, thetas_deg, m_max=m_max)
    res = prob.sweep(precision, keep=True)
    F = res.dF.sum(0)
    return prob, res, F, Bsp


def _bspline_gradient(prob, res, F, Bsp, n_radii: int, pol: str, h: float) -> np.ndarray:
    sg = ShapeGradient(prob, res, F, pol, h=h)
    grad = np.empty(n_radii)
    for j in range(n_radii):
        dn = np.zeros((prob.Nn, 2))
        dn[:, 0] = Bsp[:, j + 1]
        dn[0, 0] = dn[-1, 0] = 0.0             # the ends stay on the axis
        grad[j] = sg.directional(dn)
    prob.torch.cuda.synchronize()
    prob.check_near_status()
    prob.check_far_status()
    return grad


def bspline_rcs_and_gradient(radii: Sequence[float], n_seg: int, freq_hz: float, thetas_deg,
                             pol: str = "HH", m_max: Optional[int] = None, precision: str = "fp32ir",
                             half_length: float = 1.0, h: float = 1e-5, timings: Optional[dict] = None):
    """J = mean_theta sigma_pol of the B-spline body and dJ/d(radii) by the adjoint."""
    import time
    t0 = time.perf_counter()
    prob, res, F, Bsp = _bspline_forward(radii, n_seg, freq_hz, thetas_deg, pol, m_max, precision,
                                         half_length)
    J = objective(F, pol)
    prob.torch.cuda.synchronize()
    t1 = time.perf_counter()
    grad = _bspline_gradient(prob, res, F, Bsp, len(radii), pol, h)
    if timings is not None:
        timings["forward_s"] = t1 - t0
        timings["gradient_s"] = time.perf_counter() - t1
    return J, grad


def _rcs_function():
    import torch

    class BsplineRcs(torch.autograd.Function):
        """J(r) = mean over thetas of sigma_pol for bodies.bspline_body(r, n_seg).
        Forward: one sweep, keeping the solution on the device.  Backward: the
        adjoint gradient, recomputing the operator change of each radius."""

        @staticmethod
        def forward(ctx, radii, n_seg, freq_hz, thetas, pol, m_max, precision):
            r = radii.detach().cpu().double().numpy()
            prob, res, F, Bsp = _bspline_forward(r, int(n_seg), float(freq_hz), thetas, pol, m_max,
                                                 precision, 1.0)
            ctx.state = (prob, res, F, Bsp, len(r), pol)
            return radii.new_tensor(objective(F, pol))

        @staticmethod
        def backward(ctx, gJ):
            prob, res, F, Bsp, nr, pol = ctx.state
            grad = _bspline_gradient(prob, res, F, Bsp, nr, pol, 1e-5)
            ctx.state = None
            g = torch.as_tensor(grad, dtype=gJ.dtype, device=gJ.device)
            return gJ * g, None, None, None, None, None, None

    return BsplineRcs


def bspline_rcs(radii, n_seg: int, freq_hz: float, thetas_deg, pol: str = "HH",
                m_max: Optional[int] = None, precision: str = "fp32ir"):
    """Differentiable objective: ``bspline_rcs(r, ...).backward()`` fills r.grad."""
    return _rcs_function().apply(radii, n_seg, freq_hz, np.asarray(thetas_deg, float), pol, m_max, precision)
