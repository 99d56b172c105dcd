"""Homogeneous penetrable bodies of revolution: per-mode PMCHWT on the GPU
(the reference's solve_bor_dielectric, bor_solver.py:1019-1095).

Unknowns per mode are J (2 Nn) and M' = M / eta0 (2 Nn); with T the EFIE
operator and P the rotated principal-value operator of each medium (exterior
e = free space, interior i):

    [ T_e + T_i            -eta0 (P_e + P_i) ] [J ]   [ <W, E_inc>      ]
    [ eta0 (P_e + P_i)     T_e + r T_i       ] [M'] = [ eta0 <W, H_inc> ],
    r = (eta0 / eta_i)^2.

Every block is a fill of the PEC and impedance paths.  The interior
problem is the same generatrix at the frequency f |m| (m the refractive index
on the reference's causal branch), whose rules set n_xi and the near tables as
the reference forms them from |k_i|.  T_i is the EFIE fill with the wave
number k_i = k0 m and the factor j k_i eta_i 2 pi, P the impedance bracket
fill (ghost_bor_far_ibc / ghost_bor_near_ibc) with unit weights and no mass
term, its source columns remapped P = [[-B_tf, B_tt], [-B_ff, B_ft]]
(n x t = phi, n x phi = -t; bor_solver.py:554-576).  A lossless medium (real
m and eta_i) takes the real-k fills; a lossy one their complex-wave-number
variants (ghost_bor_*_ck, csrc/medium.cuh).  The right-hand side and the far field
come from the exterior EFIE excitation alone: the H-field excitation is the
E-field excitation of the other polarisation over eta0 (bor_solver.py:647-657),
so the columns are VV: [V_VV; -V_HH], HH: [V_HH; V_VV], and these same columns
are the reciprocity vectors of the far field of J and M together:
F_theta = c sum D (B_VV . x), F_phi = -c sum D (B_HH . x), D = diag(I, -I, I,
-I), c = -j k0 eta0 / (4 pi) -- two ghost_bor_farfield calls, one per half.
Z(-m) = S Z(m) S with S = diag(I, -I, -I, I) and B(-m) = +-S B(m), so only
m >= 0 is factored and m > 0 counts twice, as for the PEC sweep.

A purely imaginary index (an evanescent interior, Re k_i = 0) raises
NotImplementedError.
"""

from __future__ import annotations

import math
import time
from typing import Callable, Optional

import numpy as np

from . import _native as nat
from .engine import BorGpuProblem, SweepResult
from .geometry import ETA0


def medium_index(eps_r, mu_r):
    """(m, eta_i): refractive index on the causal branch (Im m <= 0, then
    Re m >= 0) and the medium's impedance eta0 mu_r / m, as the reference forms
    them (bor_solver.py:161-172).  A medium whose wave number has no real part
    (Re m = 0, an evanescent interior) raises NotImplementedError."""
    eps, mu = complex(eps_r), complex(mu_r)
    if not all(math.isfinite(v) for v in (eps.real, eps.imag, mu.real, mu.imag)):
        raise ValueError("eps_r and mu_r must be finite")
    m = complex(np.sqrt(eps * mu))
    if m.imag > 0.0:
        m = -m
    if m.real < 0.0:
        m = -m
    if not m.real > 0.0:
        raise NotImplementedError("a medium with a purely imaginary refractive index (evanescent interior) "
                                  "is not on the GPU path")
    return m, ETA0 * (mu / m)


def solve_fp64(Z, X, stream: int):
    """X <- Z^-1 X for every mode (ghost_bor_getrf / getrs, FP64; Z is
    overwritten by its factors).  Returns the per-mode LU info."""
    import torch
    Mb, n, nrhs = X.shape
    ipiv = torch.empty((Mb, n), dtype=torch.int32, device=Z.device)
    info = torch.empty((Mb,), dtype=torch.int32, device=Z.device)
    nat.call("ghost_bor_getrf", nat.F64, Mb, n, nat.ptr(Z), n, Z.stride(0), nat.ptr(ipiv),
             nat.ptr(info), 0, stream)
    nat.call("ghost_bor_getrs", nat.F64, Mb, n, nrhs, nat.ptr(Z), n, Z.stride(0), nat.ptr(ipiv),
             nat.ptr(X), nrhs, X.stride(0), 0, stream)
    return info


def residual_fp64(Z, X, B, stream: int):
    """[M+1, 2] (||Z X - B||^2, ||B||^2) per mode (ghost_bor_residual64)."""
    import torch
    Mb, n, nrhs = X.shape
    norms = torch.empty((Mb, 2), dtype=torch.float64, device=Z.device)
    nat.call("ghost_bor_residual64", Mb, n, nrhs, nat.ptr(Z), n, Z.stride(0), nat.ptr(X),
             nat.ptr(B), nrhs, B.stride(0), 0, nat.ptr(norms), stream)
    return norms


def farfield_fp64(prob: BorGpuProblem, V, X, stream: int):
    """[M+1, 2 n_theta] far-field contributions c wt sgn sum D (V . X) of a
    2 Nn row block (ghost_bor_farfield; V and X may be row blocks of larger
    systems)."""
    import torch
    Mb, n, nrhs = X.shape
    dF = torch.empty((Mb, nrhs), dtype=torch.complex128, device=X.device)
    nat.call("ghost_bor_farfield", nat.F64, Mb, n, nrhs, prob.Nn, prob.k, nat.ptr(prob.d_mode_w),
             nat.ptr(V), V.stride(-2), V.stride(0), nat.ptr(X), X.stride(-2), X.stride(0), nat.ptr(dF),
             stream)
    return dF


class DielectricBorProblem:
    """One homogeneous body at one frequency: the exterior problem (free
    space) and the interior one (the same generatrix at f |m|), with their
    tables on the device."""

    def __init__(self, points, freq_hz: float, thetas_deg, eps_r, mu_r=1.0,
                 m_max: Optional[int] = None):
        self.m_index, self.eta_i = medium_index(eps_r, mu_r)
        # a real index and impedance: the real-k fills (also a double-negative medium)
        self.lossless = self.m_index.imag == 0.0 and self.eta_i.imag == 0.0
        self.n_index = self.m_index.real if self.lossless else abs(self.m_index)
        self.eps_r, self.mu_r = complex(eps_r), complex(mu_r)
        # unit Z_s: the bracket tables and unit source weights for P.  The
        # interior problem is the generatrix at f |m|: its n_xi and near tables
        # follow |k_i|; a lossy medium's fills take the complex k_i = k0 m
        self.ext = BorGpuProblem(points, freq_hz, thetas_deg, m_max=m_max, zs=1.0)
        self.int = BorGpuProblem(points, float(freq_hz) * self.n_index, thetas_deg,
                                 m_max=self.ext.m_max, zs=1.0)
        self.k_int = self.ext.k * self.m_index
        self.m_max = self.ext.m_max
        self.Nn = self.ext.Nn
        self.n = 2 * self.ext.n           # 4 Nn unknowns per mode
        self.torch = self.ext.torch

    def bytes_needed(self) -> int:
        Mb, n, nrhs = self.m_max + 1, self.n, self.ext.nrhs
        return Mb * (2 * n * n * 16 + (n // 2) ** 2 * 16 + 3 * n * nrhs * 16)

    def keep_mask(self):
        """[M+1, 4 Nn] 1 for the unknowns each mode keeps, 0 for the masked
        J and M' rows at the axis ends (bor_solver.py:611-622, tiled twice)."""
        keep = np.ones((self.m_max + 1, self.n))
        half = self.n // 2
        for m, rows in enumerate(self.ext.masks):
            for r in rows:
                if r >= 0:
                    keep[m, r] = keep[m, r + half] = 0.0
        return keep

    def fill_system(self, stream: int):
        """The masked 4 Nn PMCHWT operator of every mode m = 0..M (FP64)."""
        torch = self.torch
        e, i = self.ext, self.int
        Mb, n, Nn = self.m_max + 1, self.n, self.Nn
        h = n // 2
        c128 = torch.complex128
        Z = torch.zeros((Mb, n, n), dtype=c128, device=e.device)
        Ce = e.C
        ki = self.k_int
        Ci = 1j * (i.k if self.lossless else ki) * self.eta_i * 2.0 * math.pi
        r2 = (ETA0 / self.eta_i) ** 2
        for blk, ci in ((Z[:, :h, :h], Ci), (Z[:, h:, h:], Ci * r2)):
            e.fill_far(blk, nat.F64, Ce, stream)
            e.fill_near(Ce, stream, Z=blk)
            if self.lossless:
                i.fill_far(blk, nat.F64, ci, stream)
                i.fill_near(ci, stream, Z=blk)
            else:
                i.fill_far_ck(blk, ki, ci, stream)
                i.fill_near_ck(ki, ci, stream, Z=blk)
        Bt = torch.zeros((Mb, h, h), dtype=c128, device=e.device)
        e.fill_far_ibc(Bt, nat.F64, 1.0 + 0.0j, stream)
        e.fill_near_ibc(1.0 + 0.0j, stream, Z=Bt, mass=False)
        if self.lossless:
            i.fill_far_ibc(Bt, nat.F64, 1.0 + 0.0j, stream)
            i.fill_near_ibc(1.0 + 0.0j, stream, Z=Bt, mass=False)
        else:
            i.fill_far_ibc_ck(Bt, ki, 1.0 + 0.0j, stream)
            i.fill_near_ibc_ck(ki, 1.0 + 0.0j, stream, Z=Bt, mass=False)
        P = ETA0 * torch.cat([-Bt[:, :, Nn:], Bt[:, :, :Nn]], dim=2)
        del Bt
        Z[:, :h, h:] -= P
        Z[:, h:, :h] += P
        del P
        keep = torch.as_tensor(self.keep_mask(), dtype=torch.float64, device=e.device)
        Z.mul_(keep[:, :, None])
        Z.mul_(keep[:, None, :])
        torch.diagonal(Z, dim1=1, dim2=2).add_(1.0 - keep)
        return Z

    def excitation(self, stream: int):
        """[M+1, 4 Nn, 2 n_theta]: VV columns [V_VV; -V_HH], HH columns
        [V_HH; V_VV] (bor_solver.py:1068-1070)."""
        torch = self.torch
        e = self.ext
        Mb, h, nrhs = self.m_max + 1, self.n // 2, e.nrhs
        V = torch.empty((Mb, h, nrhs), dtype=torch.complex128, device=e.device)
        self._rhs_work = e.excitation(V, 1.0, 0.0, stream)
        B = torch.empty((Mb, self.n, nrhs), dtype=torch.complex128, device=e.device)
        B[:, :h] = V
        B[:, h:, 0::2] = -V[:, :, 1::2]
        B[:, h:, 1::2] = V[:, :, 0::2]
        return B

    def sweep(self, check_abort: Optional[Callable] = None) -> SweepResult:
        torch = self.torch
        e = self.ext
        free, _ = torch.cuda.mem_get_info(e.device)
        free += torch.cuda.memory_reserved(e.device) - torch.cuda.memory_allocated(e.device)
        need = self.bytes_needed()
        if need > 0.92 * free:
            raise MemoryError(f"GPU sweep needs {need / 1e9:.1f} GB, {free / 1e9:.1f} GB free")
        st = nat.stream_handle()
        Mb, h = self.m_max + 1, self.n // 2
        t0 = time.perf_counter()
        Z = self.fill_system(st)
        if check_abort is not None:
            check_abort()
        Zc = Z.clone()
        B = self.excitation(st)
        X = B.clone()
        info = solve_fp64(Z, X, st)
        norms = residual_fp64(Zc, X, B, st)
        del Zc, Z
        # far field of J (top half) and M' (bottom half), each with its own
        # rows of the excitation as the reciprocity vector
        dF = farfield_fp64(e, B[:, :h], X[:, :h], st) + farfield_fp64(e, B[:, h:], X[:, h:], st)
        dF_h = dF.cpu().numpy().reshape(Mb, e.T, 2).transpose(0, 2, 1)
        res = torch.sqrt(norms[:, 0] / torch.clamp(norms[:, 1], min=1e-300)).cpu().numpy()
        info_h = info.cpu().numpy()
        e.check_near_status()
        self.int.check_near_status()
        return SweepResult(dF=np.ascontiguousarray(dF_h), residual=res, refine_iters=0,
                           timings={"wall_s": time.perf_counter() - t0}, info=info_h)
