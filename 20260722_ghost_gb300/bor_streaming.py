"""Drop-in replacement for the reference module ``bor_streaming``.

``StreamingFarBlocks`` keeps its constructor signature and per-mode accessors
(bor_streaming.py:119-421) but the far blocks of every mode are produced in one
GPU sweep by the fused far-fill kernels (ghost_bor_far_efie,
ghost_bor_far_mfie) instead of tile-by-tile CPU sampling + FFT + einsum.
``efie_blocks(m)`` returns the four nodal EFIE blocks WITHOUT the
C = j k eta 2 pi factor, ``bracket_blocks("mfie", m)`` the four MFIE
bracket blocks K (2 pi Galerkin factor included, no mass term) and
``bracket_blocks("ibc", m)`` the four rotated principal-value blocks B with
the surface impedance in the source weights (ghost_bor_far_ibc), exactly as
the reference (same/adjacent element pairs contribute zero; the near path adds
them).  Blocks are held on the device; accessors copy one mode to the host.
"""

from __future__ import annotations

from typing import Optional

import numpy as np

from . import _native as nat
from .engine import BorGpuProblem


def estimate_streaming_gb(n_elems: int, m_max: int, formulation: str = "cfie",
                          has_ibc: bool = False, single_blocks: bool = False) -> float:
    """Persistent per-mode nodal block memory of the reference's streaming
    path (bor_streaming.py:424-435)."""
    Nn = float(n_elems + 1)
    per = 8.0 if single_blocks else 16.0
    total = 4.0 * Nn * Nn * (m_max + 1) * per
    if formulation in ("cfie", "mfie"):
        total += 4.0 * Nn * Nn * (2 * m_max + 1) * per
    if has_ibc:
        total += 4.0 * Nn * Nn * (2 * m_max + 1) * per
    return total / 1e9


class StreamingFarBlocks:
    """Per-mode nodal far blocks of one surface, built on the GPU."""

    def __init__(self, solver, m_max: int, efie: bool = True, mfie: bool = False,
                 ibc_zs_pt: Optional[np.ndarray] = None, dtype=np.complex128,
                 tile_budget_gb: float = 1.0, workers: int = 1,
                 mode_block: Optional[int] = None):
        import torch
        if getattr(solver, "_lossy", False):
            raise NotImplementedError("streamed far blocks of a lossy medium are not on the GPU path "
                                      "(its operators come from assemble_mode / assemble_pmchwt_P)")
        self.solver = solver
        self.m_max = int(m_max)
        self.dtype = dtype
        self.Nn = solver.Nn
        self.mode_block = self.m_max + 1
        self.n_sweeps = 1
        self.lo, self.hi = 0, self.m_max
        # the operators of the solver's medium: its generatrix at f n
        f = solver.freq_hz * getattr(solver, "_n_index", 1.0)
        prob = BorGpuProblem(solver._points, f, (0.0,), m_max=self.m_max,
                             gauss_order=solver.gauss_order, formulation="mfie" if mfie else "efie")
        single = np.dtype(dtype) == np.complex64
        prec = nat.F32 if single else nat.F64
        self.Z = self.K = self.B = None
        if ibc_zs_pt is not None:
            # Z_s per element (constant on each element, as solve_bor builds it)
            ze = solver._zs_elem(ibc_zs_pt)
            B = torch.zeros((self.m_max + 1, prob.n, prob.n), dtype=torch.complex128, device=prob.device)
            if np.any(ze != 0.0):
                bprob = BorGpuProblem(solver._points, f, (0.0,), m_max=self.m_max,
                                      gauss_order=solver.gauss_order, zs=ze)
                bprob.fill_far_ibc(B, prec, 1.0 + 0.0j, nat.stream_handle())
            self.B = B
        if efie:
            Z = torch.zeros((self.m_max + 1, prob.n, prob.n), dtype=torch.complex128, device=prob.device)
            prob.fill_far(Z, prec, 1.0 + 0.0j, nat.stream_handle())
            self.Z = Z
        if mfie:
            # the kernel adds -scale * K (the far part of M/2 - K): scale -1 stores K
            K = torch.zeros((self.m_max + 1, prob.n, prob.n), dtype=torch.complex128, device=prob.device)
            prob.fill_far_mfie(K, prec, -1.0 + 0.0j, nat.stream_handle())
            self.K = K

    def _blocks(self, store, m: int):
        am = abs(m)
        if am > self.m_max:
            raise ValueError(f"mode {m} outside the built range 0..{self.m_max}")
        Nn = self.Nn
        Zm = store[am].cpu().numpy()
        if np.dtype(self.dtype) == np.complex64:
            Zm = Zm.astype(np.complex64).astype(np.complex128)
        ztt, ztf = Zm[:Nn, :Nn].copy(), Zm[:Nn, Nn:].copy()
        zft, zff = Zm[Nn:, :Nn].copy(), Zm[Nn:, Nn:].copy()
        if m < 0:
            ztf, zft = -ztf, -zft
        return ztt, ztf, zft, zff

    def efie_blocks(self, m: int):
        """Far EFIE blocks of mode m (bor_streaming.py:388-407)."""
        if self.Z is None:
            raise ValueError("EFIE blocks were not built")
        return self._blocks(self.Z, m)

    def bracket_blocks(self, which: str, m: int):
        """Far bracket blocks (tt, tf, ft, ff) of mode m, ``which`` = "mfie"
        (K) or "ibc" (B, Z_s in the source weights) (bor_streaming.py:409-414);
        both obey X(-m) = D X(m) D."""
        if which not in ("mfie", "ibc"):
            raise ValueError(f"unknown bracket kind {which!r}")
        store = self.K if which == "mfie" else self.B
        if store is None:
            raise ValueError(f"{which.upper()} bracket blocks were not built")
        return self._blocks(store, m)

    def memory_gb(self) -> float:
        return float(sum(t.numel() * t.element_size() for t in (self.Z, self.K, self.B)
                         if t is not None)) / 1e9
