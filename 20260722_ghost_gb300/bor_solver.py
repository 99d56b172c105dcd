"""Drop-in replacement for the reference module ``bor_solver`` (PEC,
surface-impedance and homogeneous dielectric bodies).

Same entry points, keyword arguments and result keys as the reference
(bor_solver.py:820-1004 ``solve_bor``, :1007 ``solve_bor_pec``, :175-708
``BorPecSolver``, :2179-2190 canonical generatrices); all numerics run on the
GPU through libghost_bor.so.  There is no CPU path: without the library or a
CUDA device every call raises.

Precision mapping of ``table_precision``:
  "double"          -> plain FP64 GPU path (far fill, LU and solves in FP64)
  "auto" / "single" -> FP32 far fill + FP32 LU, FP64 near/self blocks, FP64
                       residual refinement per mode (at most 5 corrections,
                       typically 3) and FP64 mode sum
``assembly``, ``workers`` and ``stream_budget_gb`` are accepted for
compatibility; the GPU fill is always a streamed (never tabulated) fill and the
memory gate is the free device memory.  ``zs`` (surface impedance, scalar or
per element) selects the IBC-EFIE as in the reference.
"""

from __future__ import annotations

import math
import time
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np

from . import _native as nat
from .bodies import cylinder_generatrix, sphere_generatrix  # noqa: F401  (reference API)
from .engine import BorGpuProblem, replay_truncation
from .geometry import (C0, ETA0, GaussData, Generatrix, basis_mask as _basis_mask,
                       default_n_modes, gauss_on_generatrix)


def estimate_bor_table_gb(n_elems: int, m_max: int, formulation: str = "cfie",
                          has_ibc: bool = False, gauss_order: int = 4,
                          single_tables: bool = False) -> float:
    """Far-table memory of the reference's table path (bor_solver.py:804-817)."""
    P = float(gauss_order * n_elems)
    per = 8.0 if single_tables else 16.0
    total = P * P * (m_max + 2) * per
    if formulation in ("cfie", "mfie"):
        total += 4.0 * P * P * (2 * m_max + 1) * per
    if has_ibc:
        total += 4.0 * P * P * (2 * m_max + 1) * per
    return total / 1e9


def _precision_of(table_precision: str) -> str:
    tp = str(table_precision).strip().lower()
    if tp not in ("auto", "single", "double"):
        raise ValueError("table_precision must be 'auto', 'single', or 'double'.")
    return "fp64" if tp == "double" else "fp32ir"


def solve_bor(points, freq_hz: float, thetas_deg, formulation: str = "efie",
              cfie_alpha: float = 0.5, zs=None, n_modes: Optional[int] = None,
              gauss_order: int = 4, mode_tol: float = 1e-6, workers: int = 1,
              progress: Optional[Callable] = None,
              check_abort: Optional[Callable] = None,
              table_precision: str = "auto", assembly: str = "auto",
              stream_budget_gb: float = 8.0) -> Dict:
    """Monostatic RCS of a body of revolution at aspect angles ``thetas_deg``
    (degrees from +z), both polarisations, on one GPU.

    Returns the reference's result dict (sigma_vv, sigma_hh, amp_vv, amp_hh,
    modes_used, n_unknowns, formulation, assembly, table_precision,
    stream_mode_block, stream_sweeps, warnings, linear_residual) plus
    ``precision``, ``refine_iters``, ``refine_residual`` and ``timings``.
    """
    t_wall = time.perf_counter()
    form = formulation.strip().lower()
    if form not in ("efie", "cfie", "mfie"):
        raise ValueError("formulation must be 'efie', 'cfie' or 'mfie'.")
    asm = str(assembly).strip().lower()
    if asm not in ("auto", "tables", "streaming"):
        raise ValueError("assembly must be 'auto', 'tables', or 'streaming'.")
    precision = _precision_of(table_precision)
    if check_abort is not None:
        check_abort()
    thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
    prob = BorGpuProblem(points, freq_hz, thetas, m_max=n_modes, gauss_order=gauss_order,
                         formulation=form, cfie_alpha=cfie_alpha, zs=zs)
    warnings = _resonance_monitor(prob, form)
    t_setup = time.perf_counter()
    res = prob.sweep(precision=precision, check_abort=check_abort)
    return _result(prob, res, thetas, form, precision, mode_tol, progress, t_wall, t_setup, warnings)


def _resonance_monitor(prob: BorGpuProblem, form: str) -> List[str]:
    """Interior-resonance guard of the reference (bor_solver.py:955-985): a
    closed body on the EFIE with a lossless (purely reactive) Z_s gets the
    per-mode condition numbers and a warning."""
    closed = prob.gen.node_on_axis(0) and prob.gen.node_on_axis(prob.Nn - 1)
    lossless = (prob.zs is not None and
                float(np.max(np.abs(np.real(prob.zs)))) < 1e-3 * float(np.max(np.abs(prob.zs))))
    prob.monitor_cond = form == "efie" and closed and lossless
    if not prob.monitor_cond:
        return []
    return ["Closed body with a lossless (purely reactive) surface impedance "
            "on the EFIE: interior cavity resonances are undamped, and "
            "results at resonant frequencies may be silently corrupted. "
            "Inspect max_cond across the frequency sweep for spikes, add "
            "loss to Z_s, or avoid closed-body reactive IBC."]


def _result(prob: BorGpuProblem, res, thetas, form: str, precision: str, mode_tol: float,
            progress: Optional[Callable], t_wall: float, t_setup: float,
            warnings: Optional[List[str]] = None) -> Dict:
    """The reference's result dict of one sweep (bor_solver.py:987-1004)."""
    F, modes_used = replay_truncation(res.dF, mode_tol)
    if progress is not None:
        progress(modes_used, prob.m_max)
    warnings = [] if warnings is None else list(warnings)
    stats: Dict = {}
    if res.cond is not None:
        conds = res.cond[: modes_used + 1]
        stats = {"max_cond": float(np.max(conds)), "median_cond": float(np.median(conds))}
        if stats["max_cond"] > 1e5:
            warnings.append(
                f"Mode-system conditioning reached {stats['max_cond']:.1e}: an "
                "interior resonance is likely at or near this frequency; the "
                "result is untrustworthy there.")
    bad = np.flatnonzero(res.info != 0)
    if bad.size:
        warnings.append(f"Zero pivot in the LU of mode(s) {bad.tolist()}: singular mode system.")
    timings = dict(res.timings)
    timings["host_setup_s"] = t_setup - t_wall
    timings["wall_s"] = time.perf_counter() - t_wall
    lin_res = float(np.max(res.residual[: modes_used + 1]))
    return {
        "theta_deg": thetas.tolist(),
        "sigma_vv": (4.0 * math.pi * np.abs(F[0]) ** 2).tolist(),
        "sigma_hh": (4.0 * math.pi * np.abs(F[1]) ** 2).tolist(),
        "amp_vv": F[0].tolist(),
        "amp_hh": F[1].tolist(),
        "modes_used": int(modes_used),
        "n_unknowns": int(prob.n),
        "formulation": form,
        "assembly": "streaming",
        "table_precision": "double" if precision == "fp64" else "single",
        "stream_mode_block": None,
        "stream_sweeps": 1,
        "warnings": warnings,
        "linear_residual": lin_res,
        "precision": precision,
        "refine_iters": int(res.refine_iters),
        "refine_residual": lin_res,
        "timings": timings,
        **stats,
    }


def solve_bor_batch(bodies, thetas_deg, formulation: str = "efie", cfie_alpha: float = 0.5,
                    mode_tol: float = 1e-6, table_precision: str = "auto",
                    progress: Optional[Callable] = None, use_graphs: bool = True,
                    autotune: bool = True) -> List[Dict]:
    """Monostatic RCS of many bodies of revolution on one GPU.

    ``bodies``: iterable of dicts with ``points``, ``freq_hz`` and optionally
    ``n_modes`` (or ``m_max``) and ``zs`` (surface impedance, as in
    solve_bor).  FP32+IR EFIE sweeps of PEC bodies run as size classes
    (batch.BorGpuBatch): the bodies of a class share one LU, one set of
    substitutions and one refinement for all their modes, and each class's
    sweep is a captured CUDA graph; the class width and the near-fill grid come
    from the autotuner's cache.  FP64, CFIE / MFIE and impedance sweeps run
    body by body,
    the next body's host set-up overlapping the current sweep.  Returns one
    ``solve_bor`` result dict per body, in order.  No counterpart in the
    reference (its callers loop over bodies).
    """
    from concurrent.futures import ThreadPoolExecutor
    form = formulation.strip().lower()
    precision = _precision_of(table_precision)
    thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
    items = list(bodies)

    def setup(b):
        t0 = time.perf_counter()
        m = b.get("n_modes", b.get("m_max"))
        prob = BorGpuProblem(b["points"], float(b["freq_hz"]), thetas, m_max=m,
                             formulation=form, cfie_alpha=cfie_alpha, zs=b.get("zs"))
        return prob, t0, time.perf_counter()

    out: List[Dict] = []
    pec = all(b.get("zs") is None or not np.any(np.abs(np.asarray(b["zs"], dtype=complex)) > 0.0)
              for b in items)
    if precision == "fp32ir" and form == "efie" and items and pec:
        from .batch import Autotuner, BorGpuBatch
        with ThreadPoolExecutor(max_workers=4) as ex:
            made = list(ex.map(setup, items))
        probs = [m[0] for m in made]
        batch = BorGpuBatch(probs, tuner=Autotuner() if autotune else None)
        results = batch.sweep(use_graphs=use_graphs)
        for i, ((prob, t0, t1), res) in enumerate(zip(made, results)):
            out.append(_result(prob, res, thetas, form, precision, mode_tol, None, t0, t1))
            if progress is not None:
                progress(i + 1, len(items))
        return out
    with ThreadPoolExecutor(max_workers=1) as ex:
        nxt = ex.submit(setup, items[0]) if items else None
        for i in range(len(items)):
            prob, t0, t1 = nxt.result()
            nxt = ex.submit(setup, items[i + 1]) if i + 1 < len(items) else None
            warnings = _resonance_monitor(prob, form)
            res = prob.sweep(precision=precision)
            out.append(_result(prob, res, thetas, form, precision, mode_tol, None, t0, t1, warnings))
            if progress is not None:
                progress(i + 1, len(items))
            del prob, res
    return out


def solve_bor_dielectric(points, freq_hz: float, thetas_deg, eps_r, mu_r=1.0,
                         n_modes: Optional[int] = None, gauss_order: int = 4,
                         mode_tol: float = 1e-6, workers: int = 1,
                         progress: Optional[Callable] = None,
                         check_abort: Optional[Callable] = None) -> Dict:
    """Monostatic RCS of a closed homogeneous penetrable body by per-mode
    PMCHWT on the GPU (bor_solver.py:1019-1095): FP64 fills, LU and far field
    of J and M; lossless media take the real-k fills, lossy ones the
    complex-k fills (a purely imaginary index raises NotImplementedError).
    Returns the reference's result dict."""
    from .penetrable import DielectricBorProblem
    t_wall = time.perf_counter()
    if gauss_order != 4:
        raise NotImplementedError("the GPU kernels are specialised for gauss_order=4")
    if check_abort is not None:
        check_abort()
    thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
    prob = DielectricBorProblem(points, freq_hz, thetas, eps_r, mu_r, m_max=n_modes)
    res = prob.sweep(check_abort=check_abort)
    F, modes_used = replay_truncation(res.dF, mode_tol)
    if progress is not None:
        progress(modes_used, prob.m_max)
    return {
        "theta_deg": thetas.tolist(),
        "sigma_vv": (4.0 * math.pi * np.abs(F[0]) ** 2).tolist(),
        "sigma_hh": (4.0 * math.pi * np.abs(F[1]) ** 2).tolist(),
        "amp_vv": F[0].tolist(),
        "amp_hh": F[1].tolist(),
        "modes_used": int(modes_used),
        "n_unknowns": int(prob.n),
        "formulation": "pmchwt",
        "eps_r": complex(eps_r),
        "mu_r": complex(mu_r),
        "linear_residual": float(np.max(res.residual[: modes_used + 1])),
        "timings": {"wall_s": time.perf_counter() - t_wall, **res.timings},
    }


def solve_bor_pec(points, freq_hz: float, thetas_deg, n_modes: Optional[int] = None,
                  gauss_order: int = 4, mode_tol: float = 1e-6) -> Dict:
    """PEC EFIE entry point (bor_solver.py:1007-1016)."""
    return solve_bor(points, freq_hz, thetas_deg, formulation="efie", n_modes=n_modes,
                     gauss_order=gauss_order, mode_tol=mode_tol)


class BorPecSolver:
    """Per-mode operator factory of one PEC surface (bor_solver.py:175-708).

    Operators are built on the GPU for all modes 0..m_max at once (FP64) and
    returned per mode as complex128 NumPy arrays for compatibility; mode -m is
    D Z(m) D for both operators.  The EFIE and MFIE operators, the mass
    blocks, the plane-wave excitations (E and H), the surface-impedance
    (IBC) operator addition, the far field with the impedance surface's
    magnetic current and the PMCHWT operator P are provided.  Z_s is per
    element (constant on each element, as solve_bor builds it).  With
    medium=(eps_r, mu_r) the operators T and P are those of that medium (a
    lossy medium's through the complex-wave-number fills; its MFIE operator
    raises NotImplementedError), the excitation and the far field stay in
    air.
    """

    def __init__(self, points, freq_hz: float, gauss_order: int = 4,
                 near_depth: int = 4, medium=None, single_tables: bool = False):
        if near_depth != 4:
            raise NotImplementedError("the GPU near kernel uses the reference's depth-4 grading")
        from .penetrable import medium_index
        # medium=(eps_r, mu_r): the operators (T, P) in that medium, i.e. of the
        # same generatrix at the frequency f |m| (whose rules set n_xi and the
        # near tables) with the wave number k0 m (complex for a lossy medium);
        # excitation and far field stay in air (bor_solver.py:175-200)
        self.freq_hz = float(freq_hz)
        self._k0 = 2.0 * math.pi * self.freq_hz / C0
        if medium is None:
            self._lossy, self._n_index, self._k_medium, self.eta = False, 1.0, self._k0, ETA0
        else:
            m_idx, eta = medium_index(*medium)
            self._lossy = not (m_idx.imag == 0.0 and eta.imag == 0.0)
            self._n_index = abs(m_idx) if self._lossy else m_idx.real
            self._k_medium = self._k0 * m_idx
            self.eta = eta if self._lossy else eta.real
        self.gen = Generatrix(np.asarray(points, dtype=float))
        self.g: GaussData = gauss_on_generatrix(self.gen, gauss_order)
        self.k = self._k_medium if self._lossy else self._k0 * self._n_index
        self.gauss_order = gauss_order
        self.near_depth = near_depth
        self.Nn = self.gen.n_nodes
        self.P = len(self.g.rho)
        T = np.zeros((self.Nn, self.P))
        D = np.zeros((self.Nn, self.P))
        idx = np.arange(self.P)
        T[self.g.elem, idx] = self.g.T0
        T[self.g.elem + 1, idx] = self.g.T1
        D[self.g.elem, idx] = self.g.dRT0
        D[self.g.elem + 1, idx] = self.g.dRT1
        self.B_T, self.B_D = T, D
        self.elem_of_pt = self.g.elem
        self._points = np.asarray(points, dtype=float)
        self._stream = None
        self._ops: Optional[Tuple[int, object]] = None
        self._mops: Optional[Tuple[int, object]] = None
        self._iops: Optional[Tuple[int, bytes, object]] = None
        self._pops: Optional[Tuple[int, object]] = None
        self._single = bool(single_tables)

    # -- operator cache ----------------------------------------------------
    def _problem(self, m_max: int, thetas=(0.0,), formulation: str = "efie", air: bool = False,
                 zs=None):
        """The GPU problem of this surface: in its medium (frequency f n), or in
        air for the excitation and the far field."""
        f = self.freq_hz if air else self.freq_hz * self._n_index
        return BorGpuProblem(self._points, f, thetas, m_max=m_max, gauss_order=self.gauss_order,
                             formulation=formulation, zs=zs)

    def enable_streaming(self, m_max: int, efie: bool = True, mfie: bool = False,
                         ibc_zs_pt: Optional[np.ndarray] = None, single_blocks: bool = False,
                         tile_budget_gb: float = 1.0, workers: int = 1,
                         mode_block: Optional[int] = None) -> None:
        from .bor_streaming import StreamingFarBlocks
        self._stream = StreamingFarBlocks(self, m_max, efie=efie, mfie=mfie, ibc_zs_pt=ibc_zs_pt,
                                          dtype=np.complex64 if single_blocks else np.complex128,
                                          tile_budget_gb=tile_budget_gb, workers=workers,
                                          mode_block=mode_block)

    def prepare_operators(self, m_max: int, efie: bool = True, mfie: bool = False,
                          ibc: bool = False, workers: int = 1) -> None:
        """Build the FP64 operators of every mode 0..m_max on the GPU
        (bor_solver.py:578-608); modes -m follow by symmetry.  The IBC
        addition depends on Z_s and is built by assemble_ibc_extra."""
        if efie and (self._ops is None or self._ops[0] < m_max):
            prob = self._problem(m_max)
            if self._lossy:
                import torch
                k = complex(self._k_medium)
                C = 1j * k * self.eta * 2.0 * math.pi
                st = nat.stream_handle()
                Z = torch.zeros((m_max + 1, prob.n, prob.n), dtype=torch.complex128, device=prob.device)
                prob.fill_far_ck(Z, k, C, st)
                prob.fill_near_ck(k, C, st, Z=Z)
                prob.check_near_status()
            else:
                Z = prob.assemble_modes_fp64()
                if self.eta != ETA0:
                    Z *= self.eta / ETA0            # C = j k eta 2 pi with this medium's eta
            self._ops = (m_max, Z)
        if mfie and self._lossy:
            raise NotImplementedError("the MFIE operator of a lossy medium is not on the GPU path")
        if mfie and (self._mops is None or self._mops[0] < m_max):
            prob = self._problem(m_max, formulation="mfie")
            self._mops = (m_max, prob.assemble_mfie_modes_fp64())

    def _mode(self, ops, m: int) -> np.ndarray:
        Z = ops[1][abs(m)].cpu().numpy()
        if m < 0:
            Nn = self.Nn
            Z[:Nn, Nn:] *= -1.0
            Z[Nn:, :Nn] *= -1.0
        return Z

    def assemble_mode(self, m: int, m_max: int) -> np.ndarray:
        """EFIE operator C [[ztt, ztf], [zft, zff]] of mode m (bor_solver.py:293-345)."""
        self.prepare_operators(max(m_max, abs(m)))
        return self._mode(self._ops, m)

    def assemble_mfie_mode(self, m: int, m_max: int) -> np.ndarray:
        """MFIE operator M/2 - K of mode m (bor_solver.py:399-435)."""
        self.prepare_operators(max(m_max, abs(m)), efie=False, mfie=True)
        return self._mode(self._mops, m)

    def _zs_elem(self, zs_pt, zs_elem=None) -> np.ndarray:
        """Z_s per element from the per-Gauss-point values (and the per-element
        array, which must agree with them)."""
        pt = np.asarray(zs_pt, dtype=complex)
        if pt.shape != (self.P,):
            raise ValueError("zs_pt must have one entry per Gauss point.")
        per = pt.reshape(self.gen.n_elems, -1)
        if np.any(per != per[:, :1]):
            raise NotImplementedError("the GPU IBC fill takes Z_s constant on each element")
        ze = per[:, 0].copy()
        if zs_elem is not None and not np.array_equal(np.asarray(zs_elem, dtype=complex), ze):
            raise ValueError("zs_pt and zs_elem disagree")
        return ze

    def assemble_ibc_extra(self, m: int, m_max: int, zs_pt: np.ndarray,
                           zs_elem: np.ndarray) -> np.ndarray:
        """IBC-EFIE addition Z_s (M/2) + B of mode m: the Z_s-weighted mass term
        plus the rotated principal-value brackets with Z_s at the source
        (bor_solver.py:534-552)."""
        ze = self._zs_elem(zs_pt, zs_elem)
        if not np.any(ze != 0.0):
            return np.zeros((2 * self.Nn, 2 * self.Nn), dtype=np.complex128)
        mm = max(m_max, abs(m))
        key = ze.tobytes()
        if self._iops is None or self._iops[0] < mm or self._iops[1] != key:
            prob = BorGpuProblem(self._points, self.freq_hz, (0.0,), m_max=mm,
                                 gauss_order=self.gauss_order, zs=ze)
            self._iops = (mm, key, prob.assemble_ibc_modes_fp64())
        return self._mode((self._iops[0], self._iops[2]), m)

    def assemble_pmchwt_P(self, m: int, m_max: int) -> np.ndarray:
        """The PMCHWT rotated principal-value operator P of mode m in this
        medium: the unit-weight IBC brackets B without mass term, source columns
        remapped P = [[-B_tf, B_tt], [-B_ff, B_ft]] (bor_solver.py:554-576)."""
        mm = max(m_max, abs(m))
        if self._pops is None or self._pops[0] < mm:
            prob = self._problem(mm, zs=1.0)
            st = nat.stream_handle()
            import torch
            B = torch.zeros((mm + 1, prob.n, prob.n), dtype=torch.complex128, device=prob.device)
            if self._lossy:
                k = complex(self._k_medium)
                prob.fill_far_ibc_ck(B, k, 1.0 + 0.0j, st)
                prob.fill_near_ibc_ck(k, 1.0 + 0.0j, st, Z=B, mass=False)
            else:
                prob.fill_far_ibc(B, nat.F64, 1.0 + 0.0j, st)
                prob.fill_near_ibc(1.0 + 0.0j, st, Z=B, mass=False)
            prob.check_near_status()
            self._pops = (mm, B)
        B = self._mode(self._pops, m)
        Nn = self.Nn
        return np.concatenate([-B[:, Nn:], B[:, :Nn]], axis=1)

    def basis_mask(self, m: int) -> np.ndarray:
        return _basis_mask(self.gen, m)

    def mass_blocks(self, weight=None) -> np.ndarray:
        """2 pi B_T diag(w rho weight) B_T^T, node-based [Nn, Nn]
        (bor_solver.py:389-397); ``weight`` per Gauss point (default 1, e.g.
        Z_s for an impedance surface).  Geometry only, like ``B_T``."""
        wgt = self.g.w * self.g.rho
        if weight is not None:
            wgt = wgt * np.asarray(weight)
        return 2.0 * np.pi * (self.B_T * wgt[None, :]) @ self.B_T.T

    # -- excitation / far field (GPU kernels, one angle) --------------------
    def _excitation(self, m: int, theta_inc_deg: float, coef_e: float, coef_h: float, h_weight=None):
        import torch
        am = abs(m)
        prob = self._problem(am, thetas=(float(theta_inc_deg),), air=True)
        prob.d_masks.fill_(-1)
        B = torch.empty((am + 1, prob.n, 2), dtype=torch.complex128, device=prob.device)
        hw = None if h_weight is None else torch.as_tensor(h_weight, dtype=torch.complex128, device=prob.device)
        prob.excitation(B, coef_e, coef_h, nat.stream_handle(), h_weight=hw)
        V = B[am].cpu().numpy()       # [2Nn, 2] (VV, HH)
        if m < 0:
            # V(-m) = D V(m) for VV and -D V(m) for HH
            Nn = self.Nn
            V[Nn:, 0] *= -1.0
            V[:Nn, 1] *= -1.0
        return V

    def rhs_mode(self, m: int, theta_inc_deg: float, pol: str) -> np.ndarray:
        """<W, E_inc> for one mode, angle and polarisation (bor_solver.py:625-645)."""
        V = self._excitation(m, theta_inc_deg, 1.0, 0.0)
        return V[:, 0 if pol.upper() in ("VV", "THETA", "TM") else 1].copy()

    def rhs_mfie_mode(self, m: int, theta_inc_deg: float, pol: str) -> np.ndarray:
        """<W, n x H_inc> rotated, for one mode, angle and polarisation
        (bor_solver.py:437-461)."""
        V = self._excitation(m, theta_inc_deg, 0.0, 1.0)
        return V[:, 0 if pol.upper() in ("VV", "THETA", "TM") else 1].copy()

    def rhs_h_mode(self, m: int, theta_inc_deg: float, pol: str) -> np.ndarray:
        """Unrotated <W, H_inc> (bor_solver.py:647-657): the incident H of one
        polarisation is the E of the other over eta0 (VV: H = -y P / eta0,
        HH: H = e_theta P / eta0), so it is rhs_mode with the pair swapped."""
        if pol.upper() in ("VV", "THETA", "TM"):
            return -self.rhs_mode(m, theta_inc_deg, "HH") / ETA0
        return self.rhs_mode(m, theta_inc_deg, "VV") / ETA0

    def farfield_mode(self, m: int, sol: np.ndarray, theta_s_deg: float,
                      zs_pt: Optional[np.ndarray] = None,
                      msol: Optional[np.ndarray] = None) -> Tuple[complex, complex]:
        """Modal far field (F_theta, F_phi) by reciprocity:
        F_theta = c (D V_VV)^T x, F_phi = -c (D V_HH)^T x, c = -j k eta0/(4 pi),
        V = V_E for a PEC current and V_E - V_H^Zs with the magnetic current
        M = -Z_s n x J of an impedance surface (equal to the reference's
        projection, bor_solver.py:659-708)."""
        if msol is not None:
            raise NotImplementedError("PMCHWT magnetic-current radiation is not on the GPU path")
        import torch
        if zs_pt is None:
            Vh = self._excitation(m, theta_s_deg, 1.0, 0.0)
        else:
            Vh = self._excitation(m, theta_s_deg, 1.0, -1.0, h_weight=self._zs_elem(zs_pt))
        V = torch.as_tensor(Vh, device="cuda")
        x = torch.as_tensor(np.asarray(sol, dtype=np.complex128), device="cuda")
        Nn = self.Nn
        d = torch.ones(2 * Nn, dtype=torch.float64, device="cuda")
        d[Nn:] = -1.0
        c = -1j * self._k0 * ETA0 / (4.0 * math.pi)
        fth = c * complex(torch.sum(d * V[:, 0] * x).cpu())
        fph = -c * complex(torch.sum(d * V[:, 1] * x).cpu())
        return fth, fph
