"""GPU sweep engine: one body, one frequency, every azimuthal mode at once.

Stages (each a C-ABI call on one CUDA stream):

  far fill      ghost_bor_far_efie_tc   alpha C Z_E far blocks, m = 0..M: FP32+IR,
                                        the azimuth transform exact on the bf16
                                        tensor cores; ghost_bor_far_efie_masked
                                        in FP64 (the comparator)
                ghost_bor_far_mfie      (1 - alpha) eta0 (-K) MFIE far brackets
                ghost_bor_far_ibc       Z_s B far brackets of an impedance surface
  near fill     ghost_bor_near_efie     near/self blocks (FP32+IR: double-float into
                                        the band; FP64: dense)
                ghost_bor_near_mfie     MFIE near brackets and the mass term M/2
                ghost_bor_near_ibc      Z_s (M/2 + B) near part of the IBC
  compose       ghost_bor_compose       A32 = fl32(Z_far + Z_near), masked
  excitation    ghost_bor_rhs           B = alpha V_E + (1 - alpha) eta0 V_H (FP64); the
                                        far-field vector separately for CFIE / MFIE
                                        (V_E) and IBC (V_E - V_H^Zs, _weighted)
  LU + solve    ghost_bor_getrf/getrs   (FP32, trailing updates on tcgen05)
  refinement    ghost_bor_residual_exact  R0 = B - (Z_far + Z_near) X0 with exact
                                        products of 8-bit slices on the bf16 tensor
                                        cores; per correction D = A32^-1 R, X += D,
                                        R -= Z D exactly for the first correction
                                        and with fl32(Z) on ghost_bor_cgemm_tc after
  far field     ghost_bor_farfield      dF[m][col] by reciprocity

Only modes m >= 0 are factored: Z(-m) = D Z(m) D with D = diag(I, -I) for the
EFIE and the MFIE operator, and the excitation obeys V(-m) = +-D V(m), so each
-m system has the solution +-D x(m) and contributes exactly the same far field;
the mode sum weights m > 0 by two (checked against the per-mode reference in
the tests).

Precisions: "fp64" is the plain FP64 path (the comparator); "fp32ir" samples
and transforms the far kernels and factors in FP32, keeps the near/self blocks,
the far-block contraction, the first residual and the mode sum in FP64-class
arithmetic, and refines each mode until its residual is below the floor or no
longer halves (at most max_refine corrections).

A surface impedance Z_s per element (IBC-EFIE) adds the impedance fills
ghost_bor_far_ibc / ghost_bor_near_ibc to the EFIE operator and takes the far
field with V_E - V_H^Zs (ghost_bor_rhs_weighted); the LU, solves and
refinement are unchanged.
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np

from . import _native as nat
from .geometry import (C0, ETA0, Generatrix, bracket_tables, dct_tables, default_n_modes,
                       element_mass, gauss_on_generatrix, mask_rows, n_xi_bracket, n_xi_efie,
                       near_tables, pack_geo)


_NEAR_SCRATCH: Dict[tuple, object] = {}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 BoR path needs a CUDA device; there is no CPU fallback")
    return torch


@dataclass
class SweepResult:
    dF: np.ndarray                 # [M+1, 2 (VV, HH), n_theta] complex128, m = 0..M (mode weight applied)
    residual: np.ndarray           # [M+1] ||AX - B|| / ||B|| per mode
    refine_iters: int
    timings: Dict[str, float] = field(default_factory=dict)
    info: Optional[np.ndarray] = None
    gpu_launches: int = 0
    res_history: List[float] = field(default_factory=list)
    # [iterations + 1, M+1] relative residual of every mode before each correction
    # and after the last (FP32+IR sweeps)
    res_history_modes: Optional[np.ndarray] = None
    # device seconds of single launches, bracketed by CUDA events on the launch stream
    kernel_s: Dict[str, List[float]] = field(default_factory=dict)
    # [M+1] 2-norm condition number of each mode's reduced system (monitor_cond)
    cond: Optional[np.ndarray] = None


class BorGpuProblem:
    """Host tables (FP64) and their device copies for one body at one frequency."""

    def __init__(self, points, freq_hz: float, thetas_deg, m_max: Optional[int] = None,
                 gauss_order: int = 4, device=None, formulation: str = "efie",
                 cfie_alpha: float = 0.5, zs=None):
        if gauss_order != 4:
            raise NotImplementedError("the GPU kernels are specialised for gauss_order=4")
        # non-finite inputs would reach the kernels' index arithmetic (tail
        # orders, n_xi); the reference lets them through to NaN results
        if not np.all(np.isfinite(np.asarray(points, dtype=float))):
            raise ValueError("generatrix nodes must be finite")
        if not np.all(np.isfinite(np.asarray(thetas_deg, dtype=float))):
            raise ValueError("aspect angles must be finite")
        if not (math.isfinite(float(freq_hz)) and float(freq_hz) > 0.0):
            raise ValueError("freq_hz must be a positive finite frequency")
        self.gen = Generatrix(points)
        self.N = self.gen.n_elems
        if self.N < 3:
            raise ValueError("the GPU path needs at least 3 generatrix elements")
        # A = alpha Z_EFIE + (1 - alpha) eta0 Z_MFIE (bor_solver.py:929-938)
        form = formulation.strip().lower()
        if form not in ("efie", "cfie", "mfie"):
            raise ValueError(f"unknown formulation {formulation!r}")
        self.formulation = form
        self.alpha = float(cfie_alpha) if form == "cfie" else (1.0 if form == "efie" else 0.0)
        # surface impedance per element (bor_solver.py:848-866): the EFIE gains
        # Z_s (M/2) + B and the far field the radiation of M = -Z_s n x J
        self.zs = impedance_per_element(zs, self.N)
        if self.zs is not None and form == "cfie":
            raise ValueError("CFIE with surface impedance is not supported in phase 2; "
                             "use formulation='efie' (lossy Z_s suppresses resonances).")
        self.ibc = self.zs is not None and self.alpha > 0.0
        torch = _torch()
        nat.load()
        self.torch = torch
        self.device = torch.device("cuda" if device is None else device)
        self.g = gauss_on_generatrix(self.gen, gauss_order)
        self.freq_hz = float(freq_hz)
        self.k = 2.0 * math.pi * self.freq_hz / C0
        self.thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
        self.rho_max = float(np.max(self.gen.nodes[:, 0]))
        if m_max is None:
            m_max = default_n_modes(self.k, self.rho_max, self.thetas)
        self.m_max = int(m_max)
        self.Nn = self.gen.n_nodes
        self.n = 2 * self.Nn
        self.P = 4 * self.N
        self.T = len(self.thetas)
        self.nrhs = 2 * self.T
        self.n_xi = n_xi_efie(self.k, self.rho_max, self.m_max)
        # the far kernels sample exp(-jkR)/R; the table carries the 1/(4 pi)
        dct, sin2 = dct_tables(self.n_xi, self.m_max + 2, scale=1.0 / (4.0 * math.pi))
        self.near = near_tables(self.gen, self.k, self.m_max)
        self.n_tail_max = int(np.max(self.near.tails[:, 1]))
        self._near_ws: Dict[str, object] = {}
        self.masks = mask_rows(self.gen, self.m_max)
        dev = self.device
        f64 = torch.float64
        elem = np.stack([self.gen.lengths, self.gen.trho, self.gen.tz])
        self.d_geo = torch.as_tensor(pack_geo(self.g), dtype=f64, device=dev)
        self.d_dct = torch.as_tensor(dct, dtype=f64, device=dev)
        self.d_dct32 = self.d_dct.to(torch.float32)            # the FP32 fill reads fl32 of the table
        self.d_sin2 = torch.as_tensor(sin2, dtype=f64, device=dev)
        self.d_nodes = torch.as_tensor(np.ascontiguousarray(self.gen.nodes), dtype=f64, device=dev)
        self.d_elem = torch.as_tensor(np.ascontiguousarray(elem), dtype=f64, device=dev)
        self.d_pairs = torch.as_tensor(self.near.pairs, dtype=torch.int32, device=dev)
        self.d_tails = torch.as_tensor(self.near.tails, dtype=torch.int32, device=dev)
        self.d_cells = torch.as_tensor(self.near.cells, dtype=f64, device=dev)
        self.d_core = torch.as_tensor(self.near.core_gl, dtype=f64, device=dev)
        self.d_tail = torch.as_tensor(self.near.tail_gl, dtype=f64, device=dev)
        self.d_masks = torch.as_tensor(self.masks, dtype=torch.int32, device=dev)
        self.d_thetas = torch.as_tensor(self.thetas, dtype=f64, device=dev)
        w = np.full(self.m_max + 1, 2.0)
        w[0] = 1.0
        self.d_mode_w = torch.as_tensor(w, dtype=f64, device=dev)
        self.C = 1j * self.k * ETA0 * 2.0 * math.pi          # bor_solver.py:338
        self.d_zs = None if self.zs is None else torch.as_tensor(self.zs, dtype=torch.complex128, device=dev)
        self.d_btab = self.d_bsin2 = self.d_emass = None
        self.n_xi_b = 0
        if self.alpha < 1.0 or self.ibc:
            self.n_xi_b = n_xi_bracket(self.k, self.rho_max, self.m_max)
            btab, bs2 = bracket_tables(self.n_xi_b, self.m_max)
            self.d_btab = torch.as_tensor(btab, dtype=f64, device=dev)
            self.d_bsin2 = torch.as_tensor(bs2, dtype=f64, device=dev)
            self.d_emass = torch.as_tensor(element_mass(self.g, self.N), dtype=f64, device=dev)
        # residual norm (relative to ||B||) where the refinement stops.  The
        # tensor-core far fill perturbs the operator by ~4e-9 of its largest
        # entries; the mode systems of closed bodies are ill-conditioned (the
        # FP32 solve is off by up to ~20% in some modes), so the residual is
        # driven well below that for the surface currents as well
        self.refine_floor = 2e-9
        # residual updates R -= Z D with exact products (the bf16-digit kernel of
        # the first residual); False: R -= fl32(Z) D on the 3xTF32 GEMM, which
        # leaves a drift (Z - fl32(Z)) (X - X0) of ~1e-8 in the residual
        self.exact_updates = True
        # with exact updates, the number of leading corrections updated exactly:
        # the first correction is the large one (up to ~20% of X in
        # ill-conditioned modes) and its drift is what matters for the far field;
        # later, small corrections take the GEMM update.  None = all exact.  At the
        # 1200-segment cone-sphere (k = 80, |m| <= 50) the default leaves ~1e-9 in
        # the far field but up to 2.0e-3 relative in single current columns of the
        # worst-conditioned mode (median 1.3e-7); refine_for_currents() settings
        # bring that column to 9.9e-5
        self.exact_update_iters = 1
        self.tensor_cores = True     # FP32 LU / solve / residual updates on tcgen05 (3xTF32)
        self.update_ws_bytes = 4 << 30   # scratch bound of one residual-update GEMM launch
        self.exact_residual = True       # first residual with exact products (bf16 Ozaki slices)
        # FP32 far fill with the azimuth transform on the bf16 tensor cores (exact
        # digit products); False selects the SIMT FP32 transform of far_fill.cu
        self.far_tc = True
        self._far_tc_ws = None
        # condition numbers of the mode systems in the sweep result (the
        # reference monitors them for closed bodies with a lossless Z_s)
        self.monitor_cond = False

    def h2d_bytes(self) -> int:
        """Bytes of host tables copied to the device for one problem."""
        return int(sum(t.numel() * t.element_size() for t in (
            self.d_geo, self.d_dct, self.d_sin2, self.d_nodes, self.d_elem, self.d_pairs,
            self.d_tails, self.d_cells, self.d_core, self.d_tail, self.d_masks, self.d_thetas,
            self.d_mode_w) + tuple(t for t in (self.d_btab, self.d_bsin2, self.d_emass, self.d_zs)
                                   if t is not None)))

    # -- memory -----------------------------------------------------------
    def bytes_needed(self, precision: str) -> int:
        Mb = self.m_max + 1
        nn = self.n * self.n
        rhs = self.n * self.nrhs
        # separate far-field vector (V_E, or V_E - V_H^Zs for an impedance surface)
        ve = Mb * rhs * 16 if (self.alpha < 1.0 or self.zs is not None) else 0
        if precision == "fp64":
            return Mb * (2 * nn * 16 + 3 * rhs * 16) + ve
        tc = 4 * 128 * Mb * (2 * self.n + 4 * max(self.n, self.nrhs)) * 2
        # Zf (c128), A (c64) and, with GEMM updates, its unfactored copy, B and
        # X (c128), the FP64 residual of the exact updates, X32 and R32 (c64),
        # the near band, LU / solve scratch and the residual-update scratch
        upd = rhs * 16 if self.exact_updates else nn * 8
        return (Mb * (nn * 16 + nn * 8 + upd + 2 * rhs * 16 + 2 * rhs * 8 + 4 * self.Nn * 5 * 16) + tc + ve
                + self.update_ws_bytes)

    # -- stages -----------------------------------------------------------
    def _far_tc_work(self, stream: int):
        """Digit planes of the DCT table for the tensor-core far fill (built once
        per problem on the device), room for the fill's double-float geometry
        words and its status word."""
        if self._far_tc_ws is None:
            lib = nat.load()
            nbytes = int(lib.ghost_bor_far_efie_tc_workspace(self.N, self.m_max, self.n_xi))
            ws = self.torch.empty(nbytes, dtype=self.torch.uint8, device=self.device)
            nat.call("ghost_bor_far_efie_tc_tables", self.m_max, self.n_xi, nat.ptr(self.d_dct),
                     nat.ptr(self.d_sin2), nat.ptr(ws), nbytes, stream)
            self._far_tc_ws = ws
        return self._far_tc_ws

    def check_far_status(self):
        if self._far_tc_ws is not None and int(self._far_tc_ws[:4].view(self.torch.int32)[0]) != 0:
            raise RuntimeError("a bounded tensor-core wait gave up in the far fill")

    def fill_far(self, Z, precision: int, scale: complex, stream: int):
        ld = Z.stride(-2)                  # row stride: Z may be a block of a larger system
        if precision == nat.F32 and self.far_tc:
            ws = self._far_tc_work(stream)
            nat.call("ghost_bor_far_efie_tc", self.N, self.m_max, self.n_xi, self.k, scale.real, scale.imag,
                     nat.ptr(self.d_geo), nat.ptr(ws), ws.numel(), nat.ptr(Z), ld, Z.stride(0), stream)
            return
        nat.call("ghost_bor_far_efie_masked", precision, self.N, self.m_max, self.n_xi, self.k,
                 scale.real, scale.imag, nat.ptr(self.d_geo), nat.ptr(self.d_dct),
                 nat.ptr(self.d_sin2), nat.ptr(Z), ld, Z.stride(0), 0,
                 nat.ptr(self.d_dct32) if precision == nat.F32 else 0, stream)

    def _near_work(self, name: str):
        """Scratch of a near kernel (azimuth nodes of every resident CTA) and
        its status word.  One buffer per device and kernel, shared by every
        problem (all launches go to one stream) and grown on demand; the
        problem keeps a reference so the buffer outlives its launches."""
        lib = nat.load()
        nbytes = int(getattr(lib, name)(self.n_tail_max))
        key = (str(self.device), name)
        work = _NEAR_SCRATCH.get(key)
        if work is None or work.numel() < nbytes:
            work = self.torch.empty(nbytes, dtype=self.torch.uint8, device=self.device)
            _NEAR_SCRATCH[key] = work
        self._near_ws[name] = work
        return work, nbytes

    def check_near_status(self):
        for name, work in self._near_ws.items():
            if int(work[:4].view(self.torch.int32)[0]) != 0:
                raise RuntimeError(f"near kernel scratch too small ({name})")

    def fill_near(self, scale: complex, stream: int, band=None, Z=None, precision: int = nat.F64):
        ld = 0 if Z is None else Z.stride(-2)
        ms = 0 if Z is None else Z.stride(0)
        work, nbytes = self._near_work("ghost_bor_near_workspace")
        nat.call("ghost_bor_near_efie", precision, self.N, self.m_max, self.k, scale.real, scale.imag,
                 nat.ptr(self.d_nodes), nat.ptr(self.d_elem), len(self.near.pairs),
                 nat.ptr(self.d_pairs), nat.ptr(self.d_tails), nat.ptr(self.d_cells),
                 self.near.cells.shape[1], nat.ptr(self.d_core), nat.ptr(self.d_tail),
                 self.near.tail_gl.shape[1], nat.ptr(band), nat.ptr(Z), ld, ms,
                 self.n_tail_max, nat.ptr(work), nbytes, stream)

    def fill_far_mfie(self, Z, precision: int, scale: complex, stream: int):
        ld = Z.stride(-2)                  # row stride: Z may be a block of a larger system
        nat.call("ghost_bor_far_mfie", precision, self.N, self.m_max, self.n_xi_b, self.k,
                 scale.real, scale.imag, nat.ptr(self.d_geo), nat.ptr(self.d_btab),
                 nat.ptr(self.d_bsin2), nat.ptr(Z), ld, Z.stride(0), stream)

    def fill_near_mfie(self, scale: complex, stream: int, band=None, Z=None):
        ld = 0 if Z is None else Z.stride(-2)
        ms = 0 if Z is None else Z.stride(0)
        work, nbytes = self._near_work("ghost_bor_near_mfie_workspace")
        nat.call("ghost_bor_near_mfie", self.N, self.m_max, self.k, scale.real, scale.imag,
                 nat.ptr(self.d_nodes), nat.ptr(self.d_elem), nat.ptr(self.d_emass),
                 len(self.near.pairs), nat.ptr(self.d_pairs), nat.ptr(self.d_tails),
                 nat.ptr(self.d_cells), self.near.cells.shape[1], nat.ptr(self.d_core),
                 nat.ptr(self.d_tail), self.near.tail_gl.shape[1], nat.ptr(band), nat.ptr(Z), ld, ms,
                 self.n_tail_max, nat.ptr(work), nbytes, stream)

    def fill_far_ibc(self, Z, precision: int, scale: complex, stream: int):
        nat.call("ghost_bor_far_ibc", precision, self.N, self.m_max, self.n_xi_b, self.k,
                 scale.real, scale.imag, nat.ptr(self.d_zs), nat.ptr(self.d_geo), nat.ptr(self.d_btab),
                 nat.ptr(self.d_bsin2), nat.ptr(Z), Z.stride(-2), Z.stride(0), stream)

    def fill_near_ibc(self, scale: complex, stream: int, band=None, Z=None, mass: bool = True):
        """Near IBC part Z_s (M/2 + B); mass=False leaves the mass term out (the
        bare brackets B, as the PMCHWT operator P takes them)."""
        ld = 0 if Z is None else Z.stride(-2)
        ms = 0 if Z is None else Z.stride(0)
        work, nbytes = self._near_work("ghost_bor_near_mfie_workspace")
        emass = self.d_emass
        if not mass:
            if getattr(self, "_zero_emass", None) is None:
                self._zero_emass = self.torch.zeros_like(self.d_emass)
            emass = self._zero_emass
        nat.call("ghost_bor_near_ibc", self.N, self.m_max, self.k, scale.real, scale.imag,
                 nat.ptr(self.d_zs), nat.ptr(self.d_nodes), nat.ptr(self.d_elem), nat.ptr(emass),
                 len(self.near.pairs), nat.ptr(self.d_pairs), nat.ptr(self.d_tails),
                 nat.ptr(self.d_cells), self.near.cells.shape[1], nat.ptr(self.d_core),
                 nat.ptr(self.d_tail), self.near.tail_gl.shape[1], nat.ptr(band), nat.ptr(Z), ld, ms,
                 self.n_tail_max, nat.ptr(work), nbytes, stream)

    # -- FP64 fills with a complex wave number (a lossy medium's interior; the
    # problem is built at the frequency of |k|, whose rules set n_xi and the
    # near tables as the reference forms them for a complex k)
    def fill_far_ck(self, Z, k: complex, scale: complex, stream: int):
        nat.call("ghost_bor_far_efie_ck", self.N, self.m_max, self.n_xi, k.real, k.imag, scale.real, scale.imag,
                 nat.ptr(self.d_geo), nat.ptr(self.d_dct), nat.ptr(self.d_sin2), nat.ptr(Z), Z.stride(-2),
                 Z.stride(0), stream)

    def fill_near_ck(self, k: complex, scale: complex, stream: int, Z=None, band=None):
        ld = 0 if Z is None else Z.stride(-2)
        ms = 0 if Z is None else Z.stride(0)
        work, nbytes = self._near_work("ghost_bor_near_workspace")
        nat.call("ghost_bor_near_efie_ck", self.N, self.m_max, k.real, k.imag, scale.real, scale.imag,
                 nat.ptr(self.d_nodes), nat.ptr(self.d_elem), len(self.near.pairs),
                 nat.ptr(self.d_pairs), nat.ptr(self.d_tails), nat.ptr(self.d_cells),
                 self.near.cells.shape[1], nat.ptr(self.d_core), nat.ptr(self.d_tail),
                 self.near.tail_gl.shape[1], nat.ptr(band), nat.ptr(Z), ld, ms,
                 self.n_tail_max, nat.ptr(work), nbytes, stream)

    def fill_far_ibc_ck(self, Z, k: complex, scale: complex, stream: int):
        nat.call("ghost_bor_far_ibc_ck", self.N, self.m_max, self.n_xi_b, k.real, k.imag,
                 scale.real, scale.imag, nat.ptr(self.d_zs), nat.ptr(self.d_geo), nat.ptr(self.d_btab),
                 nat.ptr(self.d_bsin2), nat.ptr(Z), Z.stride(-2), Z.stride(0), stream)

    def fill_near_ibc_ck(self, k: complex, scale: complex, stream: int, Z=None, band=None,
                         mass: bool = True):
        ld = 0 if Z is None else Z.stride(-2)
        ms = 0 if Z is None else Z.stride(0)
        work, nbytes = self._near_work("ghost_bor_near_mfie_workspace")
        emass = self.d_emass
        if not mass:
            if getattr(self, "_zero_emass", None) is None:
                self._zero_emass = self.torch.zeros_like(self.d_emass)
            emass = self._zero_emass
        nat.call("ghost_bor_near_ibc_ck", self.N, self.m_max, k.real, k.imag, scale.real, scale.imag,
                 nat.ptr(self.d_zs), nat.ptr(self.d_nodes), nat.ptr(self.d_elem), nat.ptr(emass),
                 len(self.near.pairs), nat.ptr(self.d_pairs), nat.ptr(self.d_tails),
                 nat.ptr(self.d_cells), self.near.cells.shape[1], nat.ptr(self.d_core),
                 nat.ptr(self.d_tail), self.near.tail_gl.shape[1], nat.ptr(band), nat.ptr(Z), ld, ms,
                 self.n_tail_max, nat.ptr(work), nbytes, stream)

    def fill_operator_far(self, Z, precision: int, stream: int):
        """Far parts of A = alpha (C Z_E + Z_s-terms) + (1 - alpha) eta0 Z_M into Z."""
        if self.alpha > 0.0:
            self.fill_far(Z, precision, self.alpha * self.C, stream)
        if self.ibc:
            # FP64 in both precisions: the refinement converges to the operator it
            # is given, and the IBC-EFIE of a closed body is far less well
            # conditioned than the CFIE, so the FP32 bracket transform's ~1e-6
            # would remain in the solution
            self.fill_far_ibc(Z, nat.F64, complex(self.alpha), stream)
        if self.alpha < 1.0:
            self.fill_far_mfie(Z, precision, complex((1.0 - self.alpha) * ETA0), stream)

    def fill_operator_near(self, stream: int, band=None, Z=None, precision: int = nat.F64):
        """Near/self parts (and the mass terms) of A into the band or Z."""
        if self.alpha > 0.0:
            self.fill_near(self.alpha * self.C, stream, band=band, Z=Z, precision=precision)
        if self.ibc:
            self.fill_near_ibc(complex(self.alpha), stream, band=band, Z=Z)
        if self.alpha < 1.0:
            self.fill_near_mfie(complex((1.0 - self.alpha) * ETA0), stream, band=band, Z=Z)

    def excitation(self, B, coef_e: float, coef_h: float, stream: int, h_weight=None):
        """B = coef_e <W, E_inc> + coef_h <W, w n x H_inc> for every mode, angle
        and polarisation; w = 1, or the complex per-element h_weight (device)."""
        torch = self.torch
        lib = nat.load()
        nbytes = int(lib.ghost_bor_rhs_workspace(self.N, self.m_max, self.T))
        work = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        if h_weight is None:
            nat.call("ghost_bor_rhs", self.N, self.m_max, self.T, self.k, coef_e, coef_h,
                     nat.ptr(self.d_geo), nat.ptr(self.d_thetas), nat.ptr(self.d_masks),
                     nat.ptr(B), B.shape[-1], B.stride(0), nat.ptr(work), stream)
        else:
            nat.call("ghost_bor_rhs_weighted", self.N, self.m_max, self.T, self.k, coef_e, coef_h,
                     nat.ptr(h_weight), nat.ptr(self.d_geo), nat.ptr(self.d_thetas), nat.ptr(self.d_masks),
                     nat.ptr(B), B.shape[-1], B.stride(0), nat.ptr(work), stream)
        return work

    def excitation_coefs(self):
        """(coef_e, coef_h) of the solve's right-hand side (bor_solver.py:939-947)."""
        return (self.alpha if self.alpha > 0.0 else 0.0,
                (1.0 - self.alpha) * ETA0 if self.alpha < 1.0 else 0.0)

    def _far_excitation(self, B, stream: int):
        """The vector the reciprocity far field dots with each solution: V_E
        (B itself for a PEC EFIE, a second excitation for CFIE / MFIE, whose B
        mixes in n x H); for an impedance surface V_E - V_H^Zs, the rotated
        n x H excitation weighted by Z_s / eta0, which adds the radiation of
        M = -Z_s n x J (bor_solver.py:659-708)."""
        if self.zs is not None:
            Ve = self.torch.empty_like(B)
            self._ve_work = self.excitation(Ve, 1.0, -1.0, stream, h_weight=self.d_zs)
            return Ve
        if self.alpha >= 1.0:
            return B
        Ve = self.torch.empty_like(B)
        self._ve_work = self.excitation(Ve, 1.0, 0.0, stream)
        return Ve

    def assemble_mfie_modes_fp64(self, stream: Optional[int] = None):
        """Dense FP64 Z_MFIE(m) = M/2 - K(m), m = 0..M, unmasked: the
        assemble_mfie_mode operator of the reference for every m >= 0."""
        torch = self.torch
        if self.d_btab is None:
            raise ValueError("this problem was built without the MFIE tables")
        st = nat.stream_handle() if stream is None else stream
        Z = torch.zeros((self.m_max + 1, self.n, self.n), dtype=torch.complex128, device=self.device)
        self.fill_far_mfie(Z, nat.F64, 1.0 + 0.0j, st)
        self.fill_near_mfie(1.0 + 0.0j, st, Z=Z)
        self.check_near_status()
        return Z

    def assemble_ibc_modes_fp64(self, stream: Optional[int] = None):
        """Dense FP64 Z_s (M/2) + B(m), m = 0..M, unmasked: the
        assemble_ibc_extra operator of the reference for every m >= 0."""
        torch = self.torch
        if self.zs is None or self.d_btab is None:
            raise ValueError("this problem was built without a surface impedance")
        st = nat.stream_handle() if stream is None else stream
        Z = torch.zeros((self.m_max + 1, self.n, self.n), dtype=torch.complex128, device=self.device)
        self.fill_far_ibc(Z, nat.F64, 1.0 + 0.0j, st)
        self.fill_near_ibc(1.0 + 0.0j, st, Z=Z)
        self.check_near_status()
        return Z

    def assemble_modes_fp64(self, stream: Optional[int] = None):
        """Dense FP64 Z(m), m = 0..M, unmasked, C factor applied: the
        assemble_mode operator of the reference for every m >= 0."""
        torch = self.torch
        st = nat.stream_handle() if stream is None else stream
        Z = torch.zeros((self.m_max + 1, self.n, self.n), dtype=torch.complex128, device=self.device)
        self.fill_operator_far(Z, nat.F64, st)
        self.fill_operator_near(st, Z=Z)
        self.check_near_status()
        return Z

    # -- the sweep ---------------------------------------------------------
    def mode_conds(self, Aop) -> np.ndarray:
        """2-norm condition number of every mode's reduced system (the rows and
        columns of its basis mask removed) from its singular values on the
        device: the figure np.linalg.cond gives the reference's monitor of
        lossless impedance surfaces (bor_solver.py:745-800).  Aop is the masked
        operator of the sweep (FP64, or its FP32 composition)."""
        torch = self.torch
        out = np.zeros(self.m_max + 1)
        for m in range(self.m_max + 1):
            drop = {int(r) for r in self.masks[m] if r >= 0}
            keep = torch.as_tensor([i for i in range(self.n) if i not in drop], device=self.device)
            A = Aop[m].index_select(0, keep).index_select(1, keep).to(torch.complex128)
            sv = torch.linalg.svdvals(A)
            out[m] = float(sv[0] / sv[-1])
        return out

    def refine_for_currents(self) -> None:
        """Refinement for surface currents within 1e-4 of the FP64 solve, not only
        the far field: every correction updates the residual with exact products
        and each mode refines down to 1e-11 of ||B||.  At the 1200-segment
        cone-sphere (k = 80, |m| <= 50) the worst current column went from 2.0e-3
        to 9.9e-5 relative and the FP32 + refinement sweep from 314 to 409 ms."""
        self.exact_update_iters = None
        self.refine_floor = 1e-11

    def sweep(self, precision: str = "fp32ir", max_refine: int = 5,
              check_abort: Optional[Callable] = None, keep: bool = False) -> SweepResult:
        torch = self.torch
        if precision not in ("fp64", "fp32ir"):
            raise ValueError("precision must be 'fp64' or 'fp32ir'")
        free, _ = torch.cuda.mem_get_info(self.device)
        # blocks cached by torch's allocator are free for this sweep too
        free += torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
        need = self.bytes_needed(precision)
        if need > 0.92 * free:
            raise MemoryError(f"GPU sweep needs {need / 1e9:.1f} GB, {free / 1e9:.1f} GB free")
        st = nat.stream_handle()
        Mb, n, nrhs, Nn = self.m_max + 1, self.n, self.nrhs, self.Nn
        ev = {}
        launches = 0

        def mark(name):
            e = torch.cuda.Event(enable_timing=True)
            e.record()
            ev[name] = e

        def abort():
            if check_abort is not None:
                check_abort()

        kev: Dict[str, list] = {}

        def kstart():
            e = torch.cuda.Event(enable_timing=True)
            e.record()
            return e

        def kend(name, e0):
            e1 = torch.cuda.Event(enable_timing=True)
            e1.record()
            kev.setdefault(name, []).append((e0, e1))

        mark("start")
        c128, c64 = torch.complex128, torch.complex64
        B = torch.empty((Mb, n, nrhs), dtype=c128, device=self.device)
        ipiv = torch.empty((Mb, n), dtype=torch.int32, device=self.device)
        info = torch.empty((Mb,), dtype=torch.int32, device=self.device)
        norms = torch.empty((Mb, 2), dtype=torch.float64, device=self.device)
        iters = 0
        history: List[float] = []
        if precision == "fp64":
            Z = torch.zeros((Mb, n, n), dtype=c128, device=self.device)
            self.fill_operator_far(Z, nat.F64, st); mark("far"); abort()
            self.fill_operator_near(st, Z=Z); mark("near")
            nat.call("ghost_bor_mask64", Mb, n, nat.ptr(self.d_masks), nat.ptr(Z), n, Z.stride(0), st)
            Zc = Z.clone()
            conds = self.mode_conds(Zc) if self.monitor_cond else None
            mark("compose"); abort()
            work = self.excitation(B, *self.excitation_coefs(), st)
            Ve = self._far_excitation(B, st); mark("rhs")
            X = B.clone()
            nat.call("ghost_bor_getrf", nat.F64, Mb, n, nat.ptr(Z), n, Z.stride(0), nat.ptr(ipiv),
                     nat.ptr(info), 0, st); mark("lu"); abort()
            nat.call("ghost_bor_getrs", nat.F64, Mb, n, nrhs, nat.ptr(Z), n, Z.stride(0), nat.ptr(ipiv),
                     nat.ptr(X), nrhs, X.stride(0), 0, st); mark("solve")
            nat.call("ghost_bor_residual64", Mb, n, nrhs, nat.ptr(Zc), n, Zc.stride(0), nat.ptr(X),
                     nat.ptr(B), nrhs, B.stride(0), 0, nat.ptr(norms), st); mark("residual")
            lu = dict(prec=nat.F64, A=Z, ipiv=ipiv, op=Zc, work=None)
            del Zc
        else:
            Zf = torch.zeros((Mb, n, n), dtype=c128, device=self.device)
            band = torch.zeros((Mb, 4, Nn, 5), dtype=c128, device=self.device)
            k0 = kstart(); self.fill_operator_far(Zf, nat.F32, st); kend("far_fill", k0)
            mark("far"); abort()
            k0 = kstart(); self.fill_operator_near(st, band=band, precision=nat.F32); kend("near_fill", k0)
            mark("near")
            A = torch.empty((Mb, n, n), dtype=c64, device=self.device)
            nat.call("ghost_bor_compose", Mb, n, Nn, nat.ptr(Zf), n, Zf.stride(0), nat.ptr(band),
                     nat.ptr(self.d_masks), nat.ptr(A), n, A.stride(0), st)
            conds = self.mode_conds(A) if self.monitor_cond else None
            mark("compose"); abort()
            work = self.excitation(B, *self.excitation_coefs(), st)
            Ve = self._far_excitation(B, st); mark("rhs")
            X32 = torch.empty((Mb, n, nrhs), dtype=c64, device=self.device)
            lib = nat.load()
            if self.tensor_cores:
                lu_ws = torch.empty(int(lib.ghost_bor_getrf_workspace(nat.F32, Mb, n)), dtype=torch.uint8,
                                    device=self.device)
                rs_ws = torch.empty(int(lib.ghost_bor_getrs_workspace(nat.F32, Mb, n, nrhs)),
                                    dtype=torch.uint8, device=self.device)
            else:
                lu_ws = rs_ws = None
            nat.call("ghost_bor_convert", 0, Mb, n, nrhs, nat.ptr(B), nrhs, B.stride(0), nat.ptr(X32),
                     nrhs, X32.stride(0), st)
            nat.call("ghost_bor_getrf", nat.F32, Mb, n, nat.ptr(A), n, A.stride(0), nat.ptr(ipiv),
                     nat.ptr(info), nat.ptr(lu_ws), st); mark("lu"); abort()
            nat.call("ghost_bor_getrs", nat.F32, Mb, n, nrhs, nat.ptr(A), n, A.stride(0), nat.ptr(ipiv),
                     nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(rs_ws), st)
            X = torch.empty((Mb, n, nrhs), dtype=c128, device=self.device)
            nat.call("ghost_bor_convert", 1, Mb, n, nrhs, nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(X),
                     nrhs, X.stride(0), st); mark("solve")
            # refinement: R0 = B - Z X0 with exact products (bf16 digit slices on
            # the tensor cores; the split-word SIMT kernel without them), Z in FP64
            # and X0 the FP32 solution; for each correction D = A^-1 R the next
            # residual is R - Z D, again with exact products (FP64 R, in place).
            # A GEMM on fl32(Z) for that product would leave the drift
            # (Z - fl32(Z)) (X - X0) in the residual, and X - X0 reaches ~20% of X
            # in ill-conditioned modes
            R32 = torch.empty((Mb, n, nrhs), dtype=c64, device=self.device)
            Ac = None
            z_split = 0
            exact_upd = self.tensor_cores and self.exact_residual and self.exact_updates
            n_exact = max_refine if self.exact_update_iters is None else min(max_refine, self.exact_update_iters)
            if (self.tensor_cores and max_refine > 0 and (not exact_upd or n_exact < max_refine)) or keep:
                # fl32(Z), masked like A, for the residual updates (and the adjoint);
                # composed before Z_far is overwritten by its FP32 words
                Ac = torch.empty((Mb, n, n), dtype=c64, device=self.device)
                nat.call("ghost_bor_compose", Mb, n, Nn, nat.ptr(Zf), n, Zf.stride(0), nat.ptr(band),
                         nat.ptr(self.d_masks), nat.ptr(Ac), n, Ac.stride(0), st)
            k0 = kstart()
            R64 = None
            if self.tensor_cores and self.exact_residual:
                # exact products on the bf16 tensor cores, modes in chunks that
                # bound the slice workspace
                per = int(lib.ghost_bor_residual_exact_workspace(1, n, nrhs))
                chunk = max(1, min(Mb, int(self.update_ws_bytes // max(per, 1))))
                ex_ws = torch.empty(int(lib.ghost_bor_residual_exact_workspace(chunk, n, nrhs)),
                                    dtype=torch.uint8, device=self.device)
                ex_flags = torch.zeros(1, dtype=torch.int32, device=self.device)
                if exact_upd and max_refine > 0:
                    R64 = torch.empty((Mb, n, nrhs), dtype=c128, device=self.device)

                def exact_residual(Xin, Bin, Rout, runs):
                    """Rout = Bin - (Z_far + Z_near) Xin (Xin FP32), norms[:, 0] = ||Rout||^2,
                    for the modes of `runs` ([b0, b1) ranges)."""
                    for r0, r1 in runs:
                        for b0 in range(r0, r1, chunk):
                            nb = min(chunk, r1 - b0)
                            nat.call("ghost_bor_residual_exact", nb, n, nrhs, Nn, nat.ptr(Zf[b0]), n, Zf.stride(0),
                                     nat.ptr(band[b0]), nat.ptr(self.d_masks[b0]), nat.ptr(Xin[b0]),
                                     nat.ptr(Bin[b0]), nrhs, Bin.stride(0),
                                     nat.ptr(None if Rout is None else Rout[b0]), nat.ptr(R32[b0]),
                                     nat.ptr(norms[b0]), nat.ptr(ex_ws), ex_ws.numel(), st)
                            torch.maximum(ex_flags, ex_ws[:4].view(torch.int32), out=ex_flags)

                exact_residual(X32, B, R64, [(0, Mb)])
            else:
                if self.tensor_cores:
                    # Z_far is read only by the first residual from here on: split it in
                    # place into FP32 words so that kernel does no FP64 work per tile
                    nat.call("ghost_bor_split_words", Mb, n, n, nat.ptr(Zf), n, Zf.stride(0), st)
                    z_split = 1
                ex_flags = None
                nat.call("ghost_bor_residual_x32", Mb, n, nrhs, Nn, nat.ptr(Zf), z_split, n, Zf.stride(0),
                         nat.ptr(band), nat.ptr(self.d_masks), nat.ptr(X32), nat.ptr(B), nrhs, B.stride(0), 0,
                         nat.ptr(R32), nat.ptr(norms), st)
            kend("residual", k0)
            bn2 = torch.clamp(norms[:, 1].clone(), min=1e-300)
            rel_d = torch.sqrt(norms[:, 0] / bn2)
            rel_m = rel_d.cpu().numpy()
            history = [float(rel_m.max())]
            hist_modes = [rel_d]
            live = np.ones(Mb, dtype=bool)
            prev_m = None
            up_ws = status = None
            for it in range(max_refine):
                # each mode stops at the residual floor or when its residual no longer
                # halves; the corrections run on the runs of modes still live
                live &= rel_m >= self.refine_floor
                if prev_m is not None:
                    live &= rel_m <= 0.5 * prev_m
                if not live.any():
                    break
                prev_m = rel_m
                runs = mode_runs(live)
                for r0, r1 in runs:
                    nb = r1 - r0
                    nat.call("ghost_bor_convert", 3, nb, n, nrhs, nat.ptr(R32[r0]), nrhs, R32.stride(0),
                             nat.ptr(X32[r0]), nrhs, X32.stride(0), st)
                    nat.call("ghost_bor_getrs", nat.F32, nb, n, nrhs, nat.ptr(A[r0]), n, A.stride(0),
                             nat.ptr(ipiv[r0]), nat.ptr(X32[r0]), nrhs, X32.stride(0), nat.ptr(rs_ws), st)
                    nat.call("ghost_bor_convert", 2, nb, n, nrhs, nat.ptr(X32[r0]), nrhs, X32.stride(0),
                             nat.ptr(X[r0]), nrhs, X.stride(0), st)
                k0 = kstart()
                if R64 is not None and it < n_exact:
                    # R -= (Z_far + Z_near) D with exact products, in FP64 (in place)
                    exact_residual(X32, R64, R64, runs)
                elif self.tensor_cores:
                    if up_ws is None:
                        per = int(lib.ghost_bor_cgemm_tc_workspace(1, n, nrhs, n))
                        chunk = max(1, min(Mb, int(self.update_ws_bytes // max(per, 1))))
                        up_ws = torch.empty(int(lib.ghost_bor_cgemm_tc_workspace(chunk, n, nrhs, n)),
                                            dtype=torch.uint8, device=self.device)
                        status = torch.zeros(1, dtype=torch.int32, device=self.device)
                    for r0, r1 in runs:
                        for b0 in range(r0, r1, chunk):
                            nb = min(chunk, r1 - b0)
                            nat.call("ghost_bor_cgemm_tc", nb, n, nrhs, n, nat.ptr(Ac[b0]), n, Ac.stride(0),
                                     nat.ptr(X32[b0]), nrhs, X32.stride(0), nat.ptr(R32[b0]), nrhs,
                                     R32.stride(0), nat.ptr(up_ws), nat.ptr(status), st)
                else:
                    # SIMT path: the split-word residual of the updated solution
                    for r0, r1 in runs:
                        Rd = torch.empty_like(B[r0:r1])
                        nat.call("ghost_bor_residual", r1 - r0, n, nrhs, Nn, nat.ptr(Zf[r0]), n, Zf.stride(0),
                                 nat.ptr(band[r0]), nat.ptr(self.d_masks[r0]), nat.ptr(X[r0]), nat.ptr(B[r0]),
                                 nrhs, B.stride(0), nat.ptr(Rd), nat.ptr(R32[r0]), nat.ptr(norms[r0]), st)
                        del Rd
                kend("residual_update", k0)
                if not (R64 is not None and it < n_exact):
                    for r0, r1 in runs:
                        norms[r0:r1, 0] = torch.linalg.vector_norm(R32[r0:r1], dim=(1, 2)).double() ** 2
                norms[:, 1].copy_(bn2)              # the kernels' second norm is of their input
                rel_d = torch.sqrt(norms[:, 0] / bn2)
                rel_m = rel_d.cpu().numpy()
                history.append(float(rel_m.max()))
                hist_modes.append(rel_d)
                iters += 1
                abort()
            if status is not None and int(status.max()) != 0:
                raise RuntimeError("a bounded tensor-core wait gave up in the residual update")
            if ex_flags is not None and int(ex_flags.max()) != 0:
                raise RuntimeError("a bounded tensor-core wait gave up in the exact residual")
            mark("residual")
            if lu_ws is not None:
                flags = torch.stack([lu_ws[:4].view(torch.int32)[0], rs_ws[:4].view(torch.int32)[0]])
                if int(flags.max()) != 0:
                    raise RuntimeError("a bounded tensor-core wait gave up in the LU / solve kernels")
            lu = dict(prec=nat.F32, A=A, ipiv=ipiv, op=Ac, work=rs_ws)
            if not keep:
                del Zf, A, Ac, R32, X32, band, R64
        dF = torch.empty((Mb, nrhs), dtype=c128, device=self.device)
        nat.call("ghost_bor_farfield", nat.F64, Mb, n, nrhs, Nn, self.k, nat.ptr(self.d_mode_w),
                 nat.ptr(Ve), nrhs, Ve.stride(0), nat.ptr(X), nrhs, X.stride(0), nat.ptr(dF), st)
        mark("farfield")
        dF_h = dF.cpu().numpy()
        res = torch.sqrt(norms[:, 0] / torch.clamp(norms[:, 1], min=1e-300)).cpu().numpy()
        info_h = info.cpu().numpy()
        torch.cuda.synchronize()
        self.check_near_status()
        self.check_far_status()
        names = list(ev)
        tm = {f"{b}_s": ev[a].elapsed_time(ev[b]) / 1e3 for a, b in zip(names[:-1], names[1:])}
        tm["gpu_total_s"] = ev[names[0]].elapsed_time(ev[names[-1]]) / 1e3
        ks = {k: [a.elapsed_time(b) / 1e3 for a, b in v] for k, v in kev.items()}
        dF_h = dF_h.reshape(Mb, self.T, 2).transpose(0, 2, 1)
        out = SweepResult(dF=np.ascontiguousarray(dF_h), residual=res, refine_iters=iters, timings=tm,
                          info=info_h, res_history=history if precision == "fp32ir" else [], kernel_s=ks,
                          res_history_modes=(torch.stack(hist_modes).cpu().numpy() if precision == "fp32ir"
                                             else None), cond=conds)
        if keep:
            out.X = X
            out.B = B
            out.Ve = Ve
            out.lu = lu          # factors, pivots and the unfactored (masked) operator
        return out


def impedance_per_element(zs, n_elem: int) -> Optional[np.ndarray]:
    """Z_s per generatrix element as the reference reads it (bor_solver.py:
    848-862): None, a complex scalar or one complex value per element; None
    when every value is zero (a PEC body)."""
    if zs is None:
        return None
    arr = np.asarray(zs, dtype=complex)
    if arr.ndim == 0:
        out = np.full(n_elem, complex(arr))
    else:
        if arr.ndim != 1 or len(arr) != n_elem:
            raise ValueError("zs array must have one entry per generatrix element.")
        out = arr.astype(complex)
    if not np.all(np.isfinite(out)):
        raise ValueError("zs must be finite")
    if np.all(np.abs(out) == 0.0):
        return None
    return np.ascontiguousarray(out)


def mode_runs(live: np.ndarray) -> List[Tuple[int, int]]:
    """[b0, b1) ranges of consecutive True entries of a per-mode mask."""
    idx = np.flatnonzero(live)
    if idx.size == 0:
        return []
    cut = np.flatnonzero(np.diff(idx) > 1)
    starts = np.concatenate([[idx[0]], idx[cut + 1]])
    ends = np.concatenate([idx[cut], [idx[-1]]]) + 1
    return [(int(a), int(b)) for a, b in zip(starts, ends)]


def replay_truncation(dF: np.ndarray, mode_tol: float):
    """The reference's mode loop in strict mode order (bor_solver.py:777-794):
    accumulate per-|m| contributions, stop after two consecutive quiet modes."""
    F = np.zeros(dF.shape[1:], dtype=np.complex128)
    quiet = 0
    used = 0
    for am in range(dF.shape[0]):
        F += dF[am]
        used = am
        scale = max(float(np.max(np.abs(F))), 1e-30)
        if float(np.max(np.abs(dF[am]))) < mode_tol * scale:
            quiet += 1
            if quiet >= 2:
                break
        else:
            quiet = 0
    return F, used
