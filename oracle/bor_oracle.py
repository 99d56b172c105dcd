"""CPU oracle for the BoR-MoM monostatic path -- TEST INFRASTRUCTURE ONLY.

A NumPy restatement of the reference's body-of-revolution solver for PEC
and surface-impedance (Leontovich, ``zs``) bodies (``bor_solver.solve_bor``
with ``formulation`` "efie" / "cfie" / "mfie", ``table_precision="double"``,
``assembly="streaming"``) and for homogeneous penetrable and coated PEC
bodies (``solve_bor_dielectric``, ``solve_bor_coated_pec``, PMCHWT).  It is the checker
that the CUDA product is compared against; the product never imports it.
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs may
import, call or time anything under ``oracle/``.

Parity pinned: ``tests/test_oracle_golden.py``, ``tests/test_oracle_ibc.py``
and ``tests/test_oracle_pmchwt.py`` check this module against golden vectors
produced by running the reference itself (``tests/golden/make_golden.py``,
``make_ibc_golden.py``, ``make_pmchwt_golden.py``).

Every function cites the reference lines it restates (paths relative to the
reference project root).  The far-field assembly follows the reference's
streaming algorithm: uniform xi sampling (C sampler ``oracle/sampler.c`` when
built, NumPy otherwise), FFT over xi, zeroing of same/adjacent-element pairs,
contraction to nodal per-order primitives (bor_streaming.py:220-407).
"""

from __future__ import annotations

import ctypes
import math
import os
import threading
from concurrent.futures import ThreadPoolExecutor
from typing import Dict, List, Optional, Tuple

import numpy as np
from scipy import special as sp

C0 = 299_792_458.0          # bor_kernels.py:29
ETA0 = 376.730313668        # bor_kernels.py:30
AXIS_TOL = 1e-12            # bor_kernels.py:31

_HERE = os.path.dirname(os.path.abspath(__file__))


# ---------------------------------------------------------------------------
# optional C sampler (oracle/sampler.c, built by oracle/build_oracle.py)
# ---------------------------------------------------------------------------

def _load_sampler():
    path = os.path.join(_HERE, "_build", "liboracle_sampler.so")
    if not os.path.exists(path):
        return None
    try:
        lib = ctypes.CDLL(path)
    except OSError:
        return None
    dp = ctypes.POINTER(ctypes.c_double)
    ci, cd = ctypes.c_int, ctypes.c_double
    lib.oracle_sample_g.argtypes = [ci, ci, ci, dp, dp, dp, dp, cd, dp, dp]
    lib.oracle_sample_g.restype = None
    lib.oracle_sample_mfie.argtypes = [ci, ci, ci] + [dp] * 8 + [cd, dp, dp] + [dp] * 4
    lib.oracle_sample_mfie.restype = None
    return lib


_SAMPLER = _load_sampler()


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# ---------------------------------------------------------------------------
# geometry: bor_kernels.py:38-125, bor_solver.py:230-242
# ---------------------------------------------------------------------------

class Geom:
    """Generatrix polyline + Gauss data (bor_kernels.py:38-82, 103-125)."""

    def __init__(self, points, gauss_order: int = 4):
        pts = np.array(points, dtype=float)
        if pts.ndim != 2 or pts.shape[1] != 2 or pts.shape[0] < 2:
            raise ValueError("Generatrix needs an (Nn, 2) array of (rho, z) nodes.")
        if np.any(pts[:, 0] < -1e-12):
            raise ValueError("Generatrix rho coordinates must be >= 0.")
        pts[:, 0] = np.maximum(pts[:, 0], 0.0)
        self.nodes = pts
        seg = pts[1:] - pts[:-1]
        self.lengths = np.hypot(seg[:, 0], seg[:, 1])
        if np.any(self.lengths <= 0):
            raise ValueError("Generatrix has a zero-length element.")
        self.trho = seg[:, 0] / self.lengths
        self.tz = seg[:, 1] / self.lengths
        self.ne = len(self.lengths)
        self.Nn = len(pts)
        # Gauss-Legendre on each element, local s in [0, 1]
        xg, wg = np.polynomial.legendre.leggauss(gauss_order)
        s = 0.5 * (xg + 1.0)
        w = 0.5 * wg
        go = gauss_order
        self.go = go
        self.elem = np.repeat(np.arange(self.ne), go)
        S = np.tile(s, self.ne)
        L = np.repeat(self.lengths, go)
        r0 = pts[:-1]
        r1 = pts[1:]
        d_rho = np.repeat(r1[:, 0] - r0[:, 0], go)
        self.s = S
        self.w = np.tile(w, self.ne) * L
        self.rho = np.repeat(r0[:, 0], go) + S * d_rho
        self.z = np.repeat(r0[:, 1], go) + S * np.repeat(r1[:, 1] - r0[:, 1], go)
        self.ptr = np.repeat(self.trho, go)
        self.ptz = np.repeat(self.tz, go)
        self.T0 = 1.0 - S
        self.T1 = S
        self.dRT0 = (d_rho * (1.0 - S) - self.rho) / L
        self.dRT1 = (d_rho * S + self.rho) / L
        self.P = len(S)
        # dense nodal shape matrices (bor_solver.py:230-242)
        self.BT = np.zeros((self.Nn, self.P))
        self.BD = np.zeros((self.Nn, self.P))
        idx = np.arange(self.P)
        self.BT[self.elem, idx] = self.T0
        self.BT[self.elem + 1, idx] = self.T1
        self.BD[self.elem, idx] = self.dRT0
        self.BD[self.elem + 1, idx] = self.dRT1

    def on_axis(self, i: int) -> bool:
        """bor_kernels.py:80-81."""
        return self.nodes[i, 0] <= AXIS_TOL * max(1.0, float(np.max(self.nodes[:, 0])))

    def points_on_element(self, e: int, s: np.ndarray):
        """bor_solver.py:117-127."""
        r0, r1 = self.nodes[e], self.nodes[e + 1]
        rho = r0[0] + s * (r1[0] - r0[0])
        z = r0[1] + s * (r1[1] - r0[1])
        L = self.lengths[e]
        drho = r1[0] - r0[0]
        d0 = (drho * (1.0 - s) - rho) / L
        d1 = (drho * s + rho) / L
        return rho, z, 1.0 - s, s, d0, d1, L


def n_xi_efie(k: float, rho_max: float, m_max: int) -> int:
    """bor_streaming.py:109-111 (= bor_kernels.py:149-152)."""
    osc = 2.0 * abs(k) * rho_max
    return int(2 ** math.ceil(math.log2(max(64, 4 * (m_max + 2), 6 * (osc + 4)))))


def n_xi_bracket(k: float, rho_max: float, m_max: int) -> int:
    """bor_streaming.py:114-116 (= bor_kernels.py:315-319)."""
    osc = 2.0 * abs(k) * rho_max
    return int(2 ** math.ceil(math.log2(max(128, 6 * (m_max + 2), 8 * (osc + 4)))))


# ---------------------------------------------------------------------------
# graded near cells: bor_solver.py:54-110
# ---------------------------------------------------------------------------

def graded_cells(kind: str, depth: int = 4) -> List[Tuple[float, float, float, float]]:
    """Quadtree of [0,1]^2 refined toward the singular set (bor_solver.py:54-78)."""
    out: List[Tuple[float, float, float, float]] = []

    def hits(a0, a1, b0, b1):
        if kind == "diag":
            return not (a1 <= b0 or b1 <= a0)
        sa = 0.0 if kind[6] == "0" else 1.0
        sb = 0.0 if kind[7] == "0" else 1.0
        return a0 <= sa <= a1 and b0 <= sb <= b1

    def split(a0, a1, b0, b1, level):
        if level >= depth or not hits(a0, a1, b0, b1):
            out.append((a0, a1, b0, b1))
            return
        am, bm = 0.5 * (a0 + a1), 0.5 * (b0 + b1)
        for (x0, x1) in ((a0, am), (am, a1)):
            for (y0, y1) in ((b0, bm), (bm, b1)):
                split(x0, x1, y0, y1, level + 1)

    split(0.0, 1.0, 0.0, 1.0, 0)
    return out


_CELLS: Dict[str, Tuple[np.ndarray, np.ndarray, np.ndarray]] = {}


def cell_points(kind: str, gorder: int = 4):
    """(s, s', weight) over the graded cells; source axis one order higher
    so test/source points never coincide (bor_solver.py:84-110)."""
    key = f"{kind}:{gorder}"
    if key not in _CELLS:
        xs, ws = np.polynomial.legendre.leggauss(gorder)
        xq, wq = np.polynomial.legendre.leggauss(gorder + 1)
        us, vs = 0.5 * (xs + 1.0), 0.5 * ws
        uq, vq = 0.5 * (xq + 1.0), 0.5 * wq
        S, Q, W = [], [], []
        for (a0, a1, b0, b1) in graded_cells(kind):
            ha, hb = a1 - a0, b1 - b0
            ss, qq = np.meshgrid(a0 + us * ha, b0 + uq * hb, indexing="ij")
            S.append(ss.ravel())
            Q.append(qq.ravel())
            W.append(np.outer(vs * ha, vq * hb).ravel())
        _CELLS[key] = (np.concatenate(S), np.concatenate(Q), np.concatenate(W))
    return _CELLS[key]


def near_kind(e: int, f: int) -> str:
    """bor_solver.py:276-282."""
    if e == f:
        return "diag"
    return "corner10" if f == e + 1 else "corner01"


# ---------------------------------------------------------------------------
# near modal kernels: bor_kernels.py:170-257, 334-431
# ---------------------------------------------------------------------------

def _near_grid(d, a, k, m_max, order=48, s0_axis=None):
    """Sinh-graded core + Gauss tail xi grid shared by the near kernels
    (bor_kernels.py:216-254, 380-404).  Returns the core's s = sin(xi/2),
    core xi / weights and tail xi / weights, each [n_pairs, n_q]."""
    s0 = np.minimum(0.25, 20.0 * d / a)
    if s0_axis is not None:
        s0 = np.where(s0_axis, 1.0, s0)
    xg, wg = np.polynomial.legendre.leggauss(order)
    u01, w01 = 0.5 * (xg + 1.0), 0.5 * wg
    vmax = np.arcsinh((a / d) * s0)
    v = u01[None, :] * vmax[:, None]
    wv = w01[None, :] * vmax[:, None]
    s = np.minimum((d / a)[:, None] * np.sinh(v), 1.0)
    xi_c = 2.0 * np.arcsin(s)
    ds_dv = (d / a)[:, None] * np.cosh(v)
    w_c = wv * 2.0 * ds_dv / np.sqrt(np.maximum(1.0 - s ** 2, 1e-15))
    osc = float(np.max(abs(complex(k)) * a)) / math.pi + (m_max + 2)
    n_tail = int(min(1024, max(64, math.ceil(4.0 * osc))))
    xt, wt = np.polynomial.legendre.leggauss(n_tail)
    xi0 = 2.0 * np.arcsin(np.minimum(s0, 1.0))
    span = np.pi - xi0
    xi_t = xi0[:, None] + 0.5 * (xt + 1.0)[None, :] * span[:, None]
    w_t = 0.5 * wt[None, :] * span[:, None]
    return s, xi_c, w_c, xi_t, w_t


def near_G(rho_p, z_p, rho_q, z_q, k, m_max, order=48):
    """G_m, m = 0..m_max+1, at near point pairs (bor_kernels.py:170-257)."""
    rho_p = np.atleast_1d(np.asarray(rho_p, float))
    rho_q = np.atleast_1d(np.asarray(rho_q, float))
    z_p = np.atleast_1d(np.asarray(z_p, float))
    z_q = np.atleast_1d(np.asarray(z_q, float))
    d2 = (rho_p - rho_q) ** 2 + (z_p - z_q) ** 2
    rr4 = 4.0 * rho_p * rho_q
    out = np.zeros((rho_p.size, m_max + 2), dtype=np.complex128)
    m = np.arange(m_max + 2)
    axis = rr4 <= 1e-30
    if np.any(axis):
        R0 = np.sqrt(d2[axis])
        out[axis, 0] = 2.0 * np.pi * np.exp(-1j * k * R0) / (4.0 * np.pi * np.maximum(R0, 1e-300))
    idx = np.flatnonzero(~axis)
    if idx.size == 0:
        return out
    d = np.sqrt(np.maximum(d2[idx], 1e-300))
    a = np.sqrt(rr4[idx])
    s_c, xi_c, w_c, xi_t, w_t = _near_grid(d, a, k, m_max, order)
    acc = np.zeros((idx.size, m_max + 2), dtype=np.complex128)
    # core: R from s directly (bor_kernels.py:228); tail: from sin(xi/2) (:248-249)
    for R, xi, w in ((np.sqrt(d[:, None] ** 2 + (a[:, None] * s_c) ** 2), xi_c, w_c),
                     (np.sqrt(d[:, None] ** 2 + (a[:, None] * np.sin(0.5 * xi_t)) ** 2), xi_t, w_t)):
        gw = np.exp(-1j * k * R) / (4.0 * np.pi * R) * w
        cm = np.cos(xi[:, :, None] * m[None, None, :])
        acc += 2.0 * (np.einsum("pv,pvm->pm", gw.real, cm)
                      + 1j * np.einsum("pv,pvm->pm", gw.imag, cm))
    out[idx, :] = acc
    return out


def _mfie_bracket_grid(rp, zp, trp, tzp, rq, zq, trq, tzq, k, xi):
    """Four MFIE brackets on per-pair xi grids (bor_kernels.py:409-426);
    test at phi = 0, source at phi' = -xi, n = (-tz, 0, tr)."""
    cx, sx = np.cos(xi), np.sin(xi)
    Rx = rp[:, None] - rq[:, None] * cx
    Ry = rq[:, None] * sx
    Rz = (zp - zq)[:, None] * np.ones_like(cx)
    R = np.maximum(np.sqrt(Rx ** 2 + Ry ** 2 + Rz ** 2), 1e-300)
    p = (1.0 + 1j * k * R) * np.exp(-1j * k * R) / (4.0 * np.pi * R ** 3)
    WtR = trp[:, None] * Rx + tzp[:, None] * Rz
    nR = -tzp[:, None] * Rx + trp[:, None] * Rz
    n_tq = -(tzp * trq)[:, None] * cx + (trp * tzq)[:, None]
    n_fq = -tzp[:, None] * sx
    Wt_tq = (trp * trq)[:, None] * cx + (tzp * tzq)[:, None]
    Wt_fq = trp[:, None] * sx
    Wf_tq = -trq[:, None] * sx
    Wf_fq = cx
    return (-p * (WtR * n_tq - Wt_tq * nR), -p * (WtR * n_fq - Wt_fq * nR),
            -p * (Ry * n_tq - Wf_tq * nR), -p * (Ry * n_fq - Wf_fq * nR))


def _ibc_bracket_grid(rp, zp, trp, tzp, rq, zq, trq, tzq, k, xi):
    """Four IBC brackets on per-pair xi grids (bor_kernels.py:449-481): the
    rotated principal-value kernel p(R) [(W_u . n_q)(R . f_v) - (W_u . f_v)
    (R . n_q)] with the SOURCE normal n_q = (-tz_q, 0, tr_q), test at
    phi = 0, source at phi' = -xi."""
    cx, sx = np.cos(xi), np.sin(xi)
    Rx = rp[:, None] - rq[:, None] * cx
    Ry = rq[:, None] * sx
    Rz = (zp - zq)[:, None] * np.ones_like(cx)
    R = np.maximum(np.sqrt(Rx ** 2 + Ry ** 2 + Rz ** 2), 1e-300)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        p = (1.0 + 1j * k * R) * np.exp(-1j * k * R) / (4.0 * np.pi * R ** 3)
        Wt_nq = -(trp * tzq)[:, None] * cx + (tzp * trq)[:, None]
        Wf_nq = tzq[:, None] * sx
        D = rp[:, None] * cx - rq[:, None]
        R_tq = trq[:, None] * D + tzq[:, None] * Rz
        R_fq = rp[:, None] * sx
        R_nq = -tzq[:, None] * D + trq[:, None] * Rz
        Wt_tq = (trp * trq)[:, None] * cx + (tzp * tzq)[:, None]
        Wt_fq = trp[:, None] * sx
        Wf_tq = -trq[:, None] * sx
        Wf_fq = cx
        return (p * (Wt_nq * R_tq - Wt_tq * R_nq), p * (Wt_nq * R_fq - Wt_fq * R_nq),
                p * (Wf_nq * R_tq - Wf_tq * R_nq), p * (Wf_nq * R_fq - Wf_fq * R_nq))


def near_mfie(rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q, k, m_max, order=48):
    """Near MFIE modal brackets for m = -m_max..m_max (bor_kernels.py:360-431)."""
    return _near_brackets(_mfie_bracket_grid, rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q,
                          k, m_max, order)


def near_ibc(rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q, k, m_max, order=48):
    """Near IBC modal brackets for m = -m_max..m_max (bor_kernels.py:509-560):
    the MFIE near grid and +-xi projection applied to the IBC brackets."""
    return _near_brackets(_ibc_bracket_grid, rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q,
                          k, m_max, order)


def _near_brackets(grid_fn, rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q, k, m_max, order):
    """Sinh-graded core + Gauss tail on xi in (0, pi], brackets at +-xi,
    projected on e^{-j m xi} (bor_kernels.py:334-357, 360-431)."""
    rho_p = np.atleast_1d(np.asarray(rho_p, float))
    rho_q = np.atleast_1d(np.asarray(rho_q, float))
    z_p = np.atleast_1d(np.asarray(z_p, float))
    z_q = np.atleast_1d(np.asarray(z_q, float))
    tr_p = np.broadcast_to(np.asarray(tr_p, float), rho_p.shape)
    tz_p = np.broadcast_to(np.asarray(tz_p, float), rho_p.shape)
    tr_q = np.broadcast_to(np.asarray(tr_q, float), rho_q.shape)
    tz_q = np.broadcast_to(np.asarray(tz_q, float), rho_q.shape)
    d2 = (rho_p - rho_q) ** 2 + (z_p - z_q) ** 2
    rr4 = 4.0 * rho_p * rho_q
    d = np.sqrt(np.maximum(d2, 1e-300))
    a = np.sqrt(np.maximum(rr4, 1e-300))
    a_safe = np.maximum(a, 1e-300)
    _, xi_c, w_c, xi_t, w_t = _near_grid(d, a_safe, k, m_max, order, s0_axis=rr4 <= 1e-30)
    # the tail order uses a (not a_safe) exactly like the reference
    xi_pos = np.concatenate([xi_c, xi_t], axis=1)
    w_pos = np.concatenate([w_c, w_t], axis=1)
    m = np.arange(-m_max, m_max + 1)
    Fp = grid_fn(rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q, k, xi_pos)
    Fm = grid_fn(rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q, k, -xi_pos)
    arg = xi_pos[:, :, None] * m[None, None, :]
    cm, sm = np.cos(arg), np.sin(arg)
    outs = []
    for fp, fm in zip(Fp, Fm):
        S = (fp + fm) * w_pos
        D = (fp - fm) * w_pos
        pc = np.einsum("pv,pvm->pm", S.real, cm) + 1j * np.einsum("pv,pvm->pm", S.imag, cm)
        ps = np.einsum("pv,pvm->pm", D.real, sm) + 1j * np.einsum("pv,pvm->pm", D.imag, sm)
        outs.append(pc - 1j * ps)
    return tuple(outs)


def causal_medium(eps_r: complex, mu_r: complex) -> Tuple[complex, complex]:
    """(refractive index m, relative impedance mu_r / m) with Im(m) <= 0 and
    Re(m) >= 0 (bor_solver.py:161-172)."""
    m = np.sqrt(complex(eps_r) * complex(mu_r))
    if m.imag > 0.0:
        m = -m
    if m.real < 0.0:
        m = -m
    return m, complex(mu_r) / m


# ---------------------------------------------------------------------------
# the solver
# ---------------------------------------------------------------------------

class OracleSolver:
    """Restatement of BorPecSolver (bor_solver.py:175-708) on the streaming
    far path (bor_streaming.py:119-421), FP64 throughout."""

    _COMBOS = (("r", "r"), ("z", "z"), ("r", "1"), ("1", "r"), ("1", "1"),
               ("d", "d"), ("d", "s"), ("s", "d"), ("s", "s"))  # bor_streaming.py:370-371

    def __init__(self, points, freq_hz: float, gauss_order: int = 4, medium=None):
        self.geo = Geom(points, gauss_order)
        k0 = 2.0 * math.pi * freq_hz / C0
        if medium is None:
            self.k, self.eta = k0, ETA0
        else:                                  # bor_solver.py:194-200
            m_idx, eta_r = causal_medium(*medium)
            self.k, self.eta = k0 * m_idx, ETA0 * eta_r
        self.freq_hz = freq_hz
        g = self.geo
        wrho = g.w * g.rho
        self.lv = {                                         # bor_streaming.py:145-152
            "r": np.stack([g.T0 * wrho * g.ptr, g.T1 * wrho * g.ptr]),
            "z": np.stack([g.T0 * wrho * g.ptz, g.T1 * wrho * g.ptz]),
            "1": np.stack([g.T0 * wrho, g.T1 * wrho]),
            "s": np.stack([g.T0 * g.w, g.T1 * g.w]),
            "d": np.stack([g.dRT0 * g.w, g.dRT1 * g.w]),
        }
        self.Zp = None      # EFIE primitives [9, M+2, Nn, Nn]
        self.Kb = None      # MFIE brackets [4, 2M+1, Nn, Nn]
        self.Bb = None      # IBC brackets, Z_s on the source side [4, 2M+1, Nn, Nn]
        self._near: Dict = {}
        self._lock = threading.Lock()

    # ---- far sampling (bor_streaming.py:320-341, 271-317) ----
    def _sample_g(self, rows: slice, n_xi: int) -> np.ndarray:
        g = self.geo
        xi = 2.0 * np.pi * np.arange(n_xi) / n_xi - np.pi
        sin2 = np.ascontiguousarray(np.sin(0.5 * xi) ** 2)
        rp = np.ascontiguousarray(g.rho[rows])
        zp = np.ascontiguousarray(g.z[rows])
        if _SAMPLER is not None and not np.iscomplexobj(self.k):
            out = np.empty((len(rp), g.P, n_xi), dtype=np.complex128)
            _SAMPLER.oracle_sample_g(len(rp), g.P, n_xi, _dp(rp), _dp(zp),
                                     _dp(np.ascontiguousarray(g.rho)),
                                     _dp(np.ascontiguousarray(g.z)), float(self.k),
                                     _dp(sin2), _dp(out))
            return out
        d2 = (rp[:, None] - g.rho[None, :]) ** 2 + (zp[:, None] - g.z[None, :]) ** 2
        rr4 = 4.0 * rp[:, None] * g.rho[None, :]
        R = np.maximum(np.sqrt(d2[..., None] + rr4[..., None] * sin2), 1e-300)
        return np.exp(-1j * self.k * R) / (4.0 * np.pi * R)

    def _sample_mfie(self, rows: slice, n_xi: int):
        g = self.geo
        xi = 2.0 * np.pi * np.arange(n_xi) / n_xi - np.pi
        nr = rows.stop - rows.start
        if _SAMPLER is not None:
            outs = tuple(np.empty((nr, g.P, n_xi), dtype=np.complex128) for _ in range(4))
            a = [np.ascontiguousarray(v[rows]) for v in (g.rho, g.z, g.ptr, g.ptz)]
            b = [np.ascontiguousarray(v) for v in (g.rho, g.z, g.ptr, g.ptz)]
            _SAMPLER.oracle_sample_mfie(nr, g.P, n_xi, *[_dp(v) for v in a],
                                        *[_dp(v) for v in b], float(self.k),
                                        _dp(np.ascontiguousarray(np.cos(xi))),
                                        _dp(np.ascontiguousarray(np.sin(xi))),
                                        *[_dp(o) for o in outs])
            return outs
        one = np.ones((nr, g.P))
        rp = (g.rho[rows][:, None] * one).ravel()
        zp = (g.z[rows][:, None] * one).ravel()
        trp = (g.ptr[rows][:, None] * one).ravel()
        tzp = (g.ptz[rows][:, None] * one).ravel()
        rq = (g.rho[None, :] * one).ravel()
        zq = (g.z[None, :] * one).ravel()
        trq = (g.ptr[None, :] * one).ravel()
        tzq = (g.ptz[None, :] * one).ravel()
        F = _mfie_bracket_grid(rp, zp, trp, tzp, rq, zq, trq, tzq, self.k,
                               np.broadcast_to(xi, (rp.size, n_xi)))
        return tuple(f.reshape(nr, g.P, n_xi) for f in F)

    def _sample_ibc(self, rows: slice, n_xi: int):
        """IBC brackets on the uniform xi grid (bor_streaming.py:296-317)."""
        g = self.geo
        xi = 2.0 * np.pi * np.arange(n_xi) / n_xi - np.pi
        nr = rows.stop - rows.start
        one = np.ones((nr, g.P))
        a = [(v[rows][:, None] * one).ravel() for v in (g.rho, g.z, g.ptr, g.ptz)]
        b = [(v[None, :] * one).ravel() for v in (g.rho, g.z, g.ptr, g.ptz)]
        F = _ibc_bracket_grid(*a, *b, self.k, np.broadcast_to(xi, (a[0].size, n_xi)))
        return tuple(f.reshape(nr, g.P, n_xi) for f in F)

    def _zero_near(self, K, e0, e1):
        """bor_streaming.py:343-349."""
        go, ne = self.geo.go, self.geo.ne
        for e in range(e0, e1):
            K[(e - e0) * go:(e - e0 + 1) * go, max(0, e - 1) * go:min(ne, e + 2) * go] = 0.0

    def _contract(self, Kn, lv_rows, rv, e0, re, out):
        """bor_streaming.py:352-368."""
        go, ne = self.geo.go, self.geo.ne
        Kr = Kn.reshape(re, go, ne, go, -1)
        L = lv_rows.reshape(2, re, go)
        R = rv.reshape(2, ne, go)
        M = np.einsum("aeg,egfhm,bfh->maebf", L, Kr, R, optimize=True)
        with self._lock:
            out[:, e0:e0 + re, 0:ne] += M[:, 0, :, 0, :]
            out[:, e0:e0 + re, 1:ne + 1] += M[:, 0, :, 1, :]
            out[:, e0 + 1:e0 + re + 1, 0:ne] += M[:, 1, :, 0, :]
            out[:, e0 + 1:e0 + re + 1, 1:ne + 1] += M[:, 1, :, 1, :]

    def _tile_elems(self, n_xi, n_arrays, workers):
        g = self.geo
        budget = 512e6 / max(1, workers)
        rows = max(g.go, int(budget / (g.P * n_xi * 16.0 * n_arrays)))
        return max(1, rows // g.go)

    def build_far(self, m_max: int, efie: bool = True, mfie: bool = False,
                  workers: int = 1, elem_range: Optional[Tuple[int, int]] = None,
                  ibc_zs_pt: Optional[np.ndarray] = None):
        """Far blocks for all orders in one sweep (bor_streaming.py:220-268).
        elem_range restricts the sweep to a slice of test elements (used only
        to time a bounded sample of the build).  ibc_zs_pt (Z_s per Gauss
        point) adds the IBC bracket blocks with Z_s in the source weights
        (bor_streaming.py:153-155, 255-258)."""
        g = self.geo
        Nn, ne, go = g.Nn, g.ne, g.go
        rho_max = float(np.max(g.nodes[:, 0]))
        nx_e = n_xi_efie(self.k, rho_max, m_max)
        nx_b = n_xi_bracket(self.k, rho_max, m_max)
        orders = np.arange(0, m_max + 2)
        ph_e = np.exp(1j * np.pi * orders) * (2.0 * np.pi / nx_e)
        ms = np.arange(-m_max, m_max + 1)
        bins = np.where(ms >= 0, ms, nx_b + ms)
        ph_b = np.exp(1j * np.pi * ms) * (2.0 * np.pi / nx_b)
        if efie:
            self.Zp = np.zeros((9, m_max + 2, Nn, Nn), dtype=np.complex128)
        if mfie:
            self.Kb = np.zeros((4, 2 * m_max + 1, Nn, Nn), dtype=np.complex128)
        ibc = ibc_zs_pt is not None
        if ibc:
            self.Bb = np.zeros((4, 2 * m_max + 1, Nn, Nn), dtype=np.complex128)
            wz = g.w * g.rho * np.asarray(ibc_zs_pt, dtype=complex)
            rv_ibc = np.stack([g.T0 * wz, g.T1 * wz])
        brk = mfie or ibc
        te = self._tile_elems(max(nx_e, nx_b if brk else 0), 6 if brk else 2, workers)
        lo, hi = (0, ne) if elem_range is None else elem_range

        def tile(e0):
            e1 = min(e0 + te, hi)
            rows = slice(e0 * go, e1 * go)
            re = e1 - e0
            if efie:
                spec = np.fft.fft(self._sample_g(rows, nx_e), axis=-1)
                Gn = spec[..., 0:m_max + 2] * ph_e
                self._zero_near(Gn, e0, e1)
                for ci, (lx, rx) in enumerate(self._COMBOS):
                    self._contract(Gn, self.lv[lx][:, rows], self.lv[rx], e0, re, self.Zp[ci])
            if mfie:
                Fs = self._sample_mfie(rows, nx_b)
                for uv, F in enumerate(Fs):
                    spec = np.fft.fft(F, axis=-1)
                    Km = spec[..., bins] * (2.0 * np.pi * ph_b)
                    self._zero_near(Km, e0, e1)
                    self._contract(Km, self.lv["1"][:, rows], self.lv["1"], e0, re, self.Kb[uv])
            if ibc:
                for uv, F in enumerate(self._sample_ibc(rows, nx_b)):
                    spec = np.fft.fft(F, axis=-1)
                    Km = spec[..., bins] * (2.0 * np.pi * ph_b)
                    self._zero_near(Km, e0, e1)
                    self._contract(Km, self.lv["1"][:, rows], rv_ibc, e0, re, self.Bb[uv])

        starts = list(range(lo, hi, te))
        if workers <= 1:
            for e0 in starts:
                tile(e0)
        else:
            with ThreadPoolExecutor(max_workers=workers) as ex:
                list(ex.map(tile, starts))

    def efie_far_blocks(self, m: int):
        """Per-mode far EFIE blocks from the primitives (bor_streaming.py:388-407)."""
        am = abs(m)
        k = self.k
        lo, hi = abs(am - 1), am + 1
        Z = self.Zp
        ztt = 0.5 * (Z[0, lo] + Z[0, hi]) + Z[1, am] - (1.0 / k ** 2) * Z[5, am]
        ztf = (Z[2, lo] - Z[2, hi]) / 2j - (1j * am / k ** 2) * Z[6, am]
        zft = -(Z[3, lo] - Z[3, hi]) / 2j + (1j * am / k ** 2) * Z[7, am]
        zff = 0.5 * (Z[4, lo] + Z[4, hi]) - (am ** 2 / k ** 2) * Z[8, am]
        if m < 0:
            ztf, zft = -ztf, -zft
        return ztt.copy(), ztf.copy(), zft.copy(), zff.copy()

    # ---- near pairs (bor_solver.py:270-290, 372-387) ----
    def near_pairs(self):
        ne = self.geo.ne
        return [(e, f) for e in range(ne) for f in (e - 1, e, e + 1) if 0 <= f < ne]

    def near_efie_data(self, e: int, f: int, m_max: int):
        key = ("efie", m_max, e, f)
        if key in self._near:
            return self._near[key]
        g = self.geo
        s, sp_, w = cell_points(near_kind(e, f))
        rp, zp, T0p, T1p, D0p, D1p, Lp = g.points_on_element(e, s)
        rq, zq, T0q, T1q, D0q, D1q, Lq = g.points_on_element(f, sp_)
        Gm = near_G(rp, zp, rq, zq, self.k, m_max)
        data = (w * Lp * Lq, rp, np.vstack([T0p, T1p]), np.vstack([D0p, D1p]),
                rq, np.vstack([T0q, T1q]), np.vstack([D0q, D1q]), Gm)
        self._near[key] = data
        return data

    def near_mfie_data(self, e: int, f: int, m_max: int):
        key = ("mfie", m_max, e, f)
        if key in self._near:
            return self._near[key]
        g = self.geo
        s, sp_, w = cell_points(near_kind(e, f))
        rp, zp, T0p, T1p, _, _, Lp = g.points_on_element(e, s)
        rq, zq, T0q, T1q, _, _, Lq = g.points_on_element(f, sp_)
        Kn = near_mfie(rp, zp, np.full_like(rp, g.trho[e]), np.full_like(rp, g.tz[e]),
                       rq, zq, np.full_like(rq, g.trho[f]), np.full_like(rq, g.tz[f]),
                       self.k, m_max)
        data = (w * Lp * Lq, rp, np.vstack([T0p, T1p]), rq, np.vstack([T0q, T1q]), Kn)
        self._near[key] = data
        return data

    def near_ibc_data(self, e: int, f: int, m_max: int):
        """bor_solver.py:481-497."""
        key = ("ibc", m_max, e, f)
        if key in self._near:
            return self._near[key]
        g = self.geo
        s, sp_, w = cell_points(near_kind(e, f))
        rp, zp, T0p, T1p, _, _, Lp = g.points_on_element(e, s)
        rq, zq, T0q, T1q, _, _, Lq = g.points_on_element(f, sp_)
        Kn = near_ibc(rp, zp, np.full_like(rp, g.trho[e]), np.full_like(rp, g.tz[e]),
                      rq, zq, np.full_like(rq, g.trho[f]), np.full_like(rq, g.tz[f]),
                      self.k, m_max)
        data = (w * Lp * Lq, rp, np.vstack([T0p, T1p]), rq, np.vstack([T0q, T1q]), Kn)
        self._near[key] = data
        return data

    def prepare(self, m_max: int, efie=True, mfie=False, workers=1,
                pairs: Optional[List[Tuple[int, int]]] = None,
                ibc_zs_pt: Optional[np.ndarray] = None):
        """Far sweep + near caches (bor_solver.py:578-608)."""
        if pairs is None:
            self.build_far(m_max, efie=efie, mfie=mfie, workers=workers, ibc_zs_pt=ibc_zs_pt)
            pairs = self.near_pairs()
        jobs = []
        if efie:
            jobs += [(self.near_efie_data, p) for p in pairs]
        if mfie:
            jobs += [(self.near_mfie_data, p) for p in pairs]
        if ibc_zs_pt is not None:
            jobs += [(self.near_ibc_data, p) for p in pairs]
        if workers <= 1:
            for fn, (e, f) in jobs:
                fn(e, f, m_max)
        else:
            with ThreadPoolExecutor(max_workers=workers) as ex:
                list(ex.map(lambda j: j[0](j[1][0], j[1][1], m_max), jobs))

    # ---- per-mode operators ----
    def assemble_efie(self, m: int, m_max: int) -> np.ndarray:
        """bor_solver.py:293-345 on streamed far blocks."""
        g = self.geo
        k = self.k
        ztt, ztf, zft, zff = self.efie_far_blocks(m)
        am = abs(m)
        for (e, f) in self.near_pairs():
            w, rp, Tp, Dp, rq, Tq, Dq, Gm = self.near_efie_data(e, f, m_max)
            Gn = Gm[:, am]
            Gc = 0.5 * (Gm[:, abs(am - 1)] + Gm[:, am + 1])
            Gs = (Gm[:, abs(am - 1)] - Gm[:, am + 1]) / 2j
            if m < 0:
                Gs = -Gs
            rr = rp * rq * w
            ktt = rr * (g.trho[e] * g.trho[f] * Gc + g.tz[e] * g.tz[f] * Gn)
            ksc = w * Gn
            ktf = rr * (g.trho[e] * Gs)
            kft = -rr * (g.trho[f] * Gs)
            kff = rr * Gc
            c = lambda A, kk, B: np.einsum("ip,p,jp->ij", A, kk, B)
            rs, cs = slice(e, e + 2), slice(f, f + 2)
            ztt[rs, cs] += c(Tp, ktt, Tq) - (1.0 / k ** 2) * c(Dp, ksc, Dq)
            ztf[rs, cs] += c(Tp, ktf, Tq) - (1j * m / k ** 2) * c(Dp, ksc, Tq)
            zft[rs, cs] += c(Tp, kft, Tq) + (1j * m / k ** 2) * c(Tp, ksc, Dq)
            zff[rs, cs] += c(Tp, kff, Tq) - (m ** 2 / k ** 2) * c(Tp, ksc, Tq)
        C = 1j * k * self.eta * 2.0 * np.pi
        return C * np.block([[ztt, ztf], [zft, zff]])

    def mass(self, weight: Optional[np.ndarray] = None) -> np.ndarray:
        """bor_solver.py:389-397 (weight: per Gauss point, e.g. Z_s)."""
        g = self.geo
        wgt = g.w * g.rho if weight is None else g.w * g.rho * np.asarray(weight)
        return 2.0 * np.pi * (g.BT * wgt[None, :]) @ g.BT.T

    def assemble_ibc_extra(self, m: int, m_max: int, zs_pt: np.ndarray,
                           zs_elem: np.ndarray) -> np.ndarray:
        """IBC-EFIE terms from eliminating M = -Z_s n x J (bor_solver.py:
        499-552): (1/2) <W, Z_s J> + the rotated principal-value brackets
        with Z_s at the source; the far part comes from build_far(ibc_zs_pt),
        near pairs are weighted by the source element's Z_s."""
        ktt, ktf, kft, kff = self.rot_pv_blocks(m, m_max, zs_elem)
        Mz = self.mass(zs_pt)
        return np.block([[0.5 * Mz + ktt, ktf], [kft, 0.5 * Mz + kff]])

    def rot_pv_blocks(self, m: int, m_max: int, zs_elem: Optional[np.ndarray] = None):
        """The four rotated principal-value blocks B_tt, B_tf, B_ft, B_ff of
        mode m with an optional source weight per element (bor_solver.py:
        497-532): far part from build_far(ibc_zs_pt = that weight per Gauss
        point, or ones), near pairs weighted by the source element's value."""
        mi = m + m_max
        blocks = [self.Bb[uv, mi].copy() for uv in range(4)]
        for (e, f) in self.near_pairs():
            welem = 1.0 if zs_elem is None else zs_elem[f]
            if abs(welem) == 0.0:
                continue
            w, rp, Tp, rq, Tq, Kn = self.near_ibc_data(e, f, m_max)
            rr = rp * rq * w * welem
            for uv in range(4):
                blocks[uv][e:e + 2, f:f + 2] += 2.0 * np.pi * np.einsum(
                    "ip,p,jp->ij", Tp, rr * Kn[uv][:, mi], Tq)
        return blocks

    def pmchwt_P(self, m: int, m_max: int) -> np.ndarray:
        """PMCHWT operator P in this medium acting on a magnetic current in the
        same (t, phi) bases: the unweighted rotated blocks with the source
        columns remapped (n x t = phi, n x phi = -t; bor_solver.py:554-576).
        Needs build_far / prepare with ibc_zs_pt = ones."""
        btt, btf, bft, bff = self.rot_pv_blocks(m, m_max)
        return np.block([[-btf, btt], [-bff, bft]])

    def assemble_mfie(self, m: int, m_max: int) -> np.ndarray:
        """Z_MFIE = M/2 - K (bor_solver.py:399-435) on streamed brackets."""
        mi = m + m_max
        blocks = [self.Kb[uv, mi].copy() for uv in range(4)]
        for (e, f) in self.near_pairs():
            w, rp, Tp, rq, Tq, Kn = self.near_mfie_data(e, f, m_max)
            rr = rp * rq * w
            for uv in range(4):
                blocks[uv][e:e + 2, f:f + 2] += 2.0 * np.pi * np.einsum(
                    "ip,p,jp->ij", Tp, rr * Kn[uv][:, mi], Tq)
        M = self.mass()
        ktt, ktf, kft, kff = blocks
        return np.block([[0.5 * M - ktt, -ktf], [-kft, 0.5 * M - kff]])

    def basis_mask(self, m: int) -> np.ndarray:
        """bor_solver.py:611-622."""
        Nn = self.geo.Nn
        t = np.ones(Nn, dtype=bool)
        f = np.ones(Nn, dtype=bool)
        for end in (0, Nn - 1):
            if self.geo.on_axis(end):
                t[end] = abs(m) == 1
                f[end] = False
            else:
                t[end] = False
                f[end] = True
        return np.concatenate([t, f])

    # ---- excitation / far field, vectorised over angles ----
    def _bessel_parts(self, m: int, thetas_deg: np.ndarray, sign: int):
        g = self.geo
        th = np.radians(thetas_deg)
        st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
        u = self.k * g.rho[None, :] * st
        P = np.exp(1j * self.k * ct * g.z[None, :])
        jm = lambda n: (1j) ** n * sp.jv(n, u)
        J0 = jm(m)
        Jlo, Jhi = jm(m - sign), jm(m + sign)
        Ic = math.pi * (Jlo + Jhi)
        Is = (math.pi / 1j) * (Jlo - Jhi)
        I1 = 2.0 * math.pi * J0
        return st, ct, P, Ic, Is, I1

    def rhs_efie(self, m: int, thetas_deg, pol: str) -> np.ndarray:
        """rhs_mode (bor_solver.py:625-645) for every angle: [n_theta, 2Nn]."""
        g = self.geo
        st, ct, P, Ic, Is, I1 = self._bessel_parts(m, np.atleast_1d(thetas_deg), 1)
        if pol == "VV":
            et = ct * g.ptr * Ic - st * g.ptz * I1
            ef = -ct * Is
        else:
            et = g.ptr * Is
            ef = Ic
        c = g.w * g.rho * P
        return np.concatenate([(c * et) @ g.BT.T, (c * ef) @ g.BT.T], axis=1)

    def rhs_mfie(self, m: int, thetas_deg, pol: str) -> np.ndarray:
        """rhs_mfie_mode (bor_solver.py:437-461) for every angle."""
        g = self.geo
        st, ct, P, Ic, Is, I1 = self._bessel_parts(m, np.atleast_1d(thetas_deg), 1)
        if pol == "VV":
            et = Ic / ETA0
            ef = -(g.ptr * Is) / ETA0
        else:
            et = (ct * Is) / ETA0
            ef = (ct * g.ptr * Ic - st * g.ptz * I1) / ETA0
        c = g.w * g.rho * P
        return np.concatenate([(c * et) @ g.BT.T, (c * ef) @ g.BT.T], axis=1)

    def farfield(self, m: int, sols: np.ndarray, thetas_deg,
                 zs_pt: Optional[np.ndarray] = None,
                 msol: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray]:
        """farfield_mode (bor_solver.py:659-708) for solution rows
        sols [n_theta, 2Nn] at the matching angles: (F_theta, F_phi).  With
        zs_pt the eliminated magnetic current M_t = Z_s J_phi,
        M_phi = -Z_s J_t radiates too (bor_solver.py:697-707)."""
        g = self.geo
        Nn = g.Nn
        st, ct, P, Icos, Isin, I1 = self._bessel_parts(m, np.atleast_1d(thetas_deg), -1)
        Jt = sols[:, :Nn] @ g.BT
        Jf = sols[:, Nn:] @ g.BT
        common = g.w * g.rho * P

        def proj_theta(Xt, Xf):
            return np.sum(common * (Xt * (ct * g.ptr * Icos - st * g.ptz * I1) + Xf * (-ct * Isin)),
                          axis=1)

        def proj_phi(Xt, Xf):
            return np.sum(common * (Xt * g.ptr * Isin + Xf * Icos), axis=1)

        pref = -1j * self.k * ETA0 / (4.0 * math.pi)
        fth, fph = pref * proj_theta(Jt, Jf), pref * proj_phi(Jt, Jf)
        Mt = Mf = None
        if zs_pt is not None:
            Mt, Mf = zs_pt * Jf, -zs_pt * Jt
        elif msol is not None:                 # a magnetic-current solution (PMCHWT)
            Mt, Mf = msol[:, :Nn] @ g.BT, msol[:, Nn:] @ g.BT
        if Mt is not None:
            pm = 1j * self.k / (4.0 * math.pi)
            fth = fth - pm * proj_phi(Mt, Mf)
            fph = fph + pm * proj_theta(Mt, Mf)
        return fth, fph


def default_n_modes(points, freq_hz: float, thetas_deg) -> int:
    """bor_solver.py:845-847."""
    pts = np.asarray(points, float)
    k = 2.0 * math.pi * freq_hz / C0
    st = float(np.max(np.abs(np.sin(np.radians(np.atleast_1d(thetas_deg))))))
    return int(math.ceil(k * float(np.max(pts[:, 0])) * max(st, 0.05))) + 12


def solve_bor(points, freq_hz: float, thetas_deg, formulation: str = "efie",
              cfie_alpha: float = 0.5, n_modes: Optional[int] = None,
              mode_tol: float = 1e-6, gauss_order: int = 4, workers: int = 1,
              keep_per_mode: bool = False, modes_subset=None,
              timings: Optional[Dict[str, float]] = None, zs=None) -> Dict:
    """Monostatic RCS (bor_solver.py:820-1004 with table_precision
    "double", assembly "streaming") and the mode loop (bor_solver.py:711-801).
    zs: None (PEC), a complex scalar or one value per element: the IBC-EFIE
    (bor_solver.py:850-864, 929-934, 947-949); the CFIE with Z_s raises.

    modes_subset (tuple of |m|) solves only those |m| -- used to time a bounded
    sample; the result then holds partial sums."""
    import time
    form = formulation.strip().lower()
    thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
    if n_modes is None:
        n_modes = default_n_modes(points, freq_hz, thetas)
    m_max = int(n_modes)
    alpha = float(cfie_alpha) if form == "cfie" else (1.0 if form == "efie" else 0.0)
    sol = OracleSolver(points, freq_hz, gauss_order)
    Nn = sol.geo.Nn
    zs_pt = zs_elem = None
    if zs is not None:
        za = np.asarray(zs, dtype=complex)
        if za.ndim == 0:
            zs_elem = np.full(sol.geo.ne, complex(za))
        elif len(za) != sol.geo.ne:
            raise ValueError("zs array must have one entry per generatrix element.")
        else:
            zs_elem = za.copy()
        zs_pt = zs_elem[sol.geo.elem]
        if np.all(np.abs(zs_pt) == 0.0):
            zs_pt = None
        elif form == "cfie":
            raise ValueError("CFIE with surface impedance is not supported; use 'efie'.")
    ibc = zs_pt is not None and alpha > 0.0
    t0 = time.perf_counter()
    sol.prepare(m_max, efie=alpha > 0.0, mfie=alpha < 1.0, workers=workers,
                ibc_zs_pt=zs_pt if ibc else None)
    t1 = time.perf_counter()
    pols = ("VV", "HH")
    F = np.zeros((2, len(thetas)), dtype=np.complex128)
    per_mode = {}

    def solve_am(am):
        dF = np.zeros_like(F)
        res = 0.0
        for m in ([0] if am == 0 else [am, -am]):
            Z = np.zeros((2 * Nn, 2 * Nn), dtype=np.complex128)
            if alpha > 0.0:
                Z += alpha * sol.assemble_efie(m, m_max)
                if ibc:
                    Z += alpha * sol.assemble_ibc_extra(m, m_max, zs_pt, zs_elem)
            if alpha < 1.0:
                Z += (1.0 - alpha) * ETA0 * sol.assemble_mfie(m, m_max)
            mask = sol.basis_mask(m)
            A = Z[np.ix_(mask, mask)]
            cols = []
            for pol in pols:
                V = np.zeros((len(thetas), 2 * Nn), dtype=np.complex128)
                if alpha > 0.0:
                    V += alpha * sol.rhs_efie(m, thetas, pol)
                if alpha < 1.0:
                    V += (1.0 - alpha) * ETA0 * sol.rhs_mfie(m, thetas, pol)
                cols.append(V)
            # column order theta-major, pol-minor (bor_solver.py:750-751)
            B = np.stack([cols[0], cols[1]], axis=1)            # [n_theta, 2, 2Nn]
            B = B.transpose(2, 0, 1).reshape(2 * Nn, 2 * len(thetas))[mask]
            X = np.linalg.solve(A, B)
            bn = float(np.linalg.norm(B))
            if bn > 0.0:
                res = max(res, float(np.linalg.norm(A @ X - B)) / bn)
            full = np.zeros((2 * Nn, X.shape[1]), dtype=np.complex128)
            full[mask] = X
            xs = full.T.reshape(len(thetas), 2, 2 * Nn)
            fth, _ = sol.farfield(m, xs[:, 0, :], thetas, zs_pt=zs_pt)
            _, fph = sol.farfield(m, xs[:, 1, :], thetas, zs_pt=zs_pt)
            dF[0] += fth
            dF[1] += fph
            if keep_per_mode:
                per_mode[m] = (A, B, X)
        return dF, res

    modes_used = 0
    quiet = 0
    max_res = 0.0
    am_list = list(range(m_max + 1)) if modes_subset is None else list(modes_subset)
    dFs = []
    with ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        results = list(ex.map(solve_am, am_list))
    for am, (dF, res) in zip(am_list, results):
        dFs.append(dF)
        if modes_subset is not None:
            F += dF
            max_res = max(max_res, res)
            modes_used = am
            continue
        F += dF
        max_res = max(max_res, res)
        modes_used = am
        scale = max(float(np.max(np.abs(F))), 1e-30)
        if float(np.max(np.abs(dF))) < mode_tol * scale:
            quiet += 1
            if quiet >= 2:
                break
        else:
            quiet = 0
    t2 = time.perf_counter()
    if timings is not None:
        timings["prepare_s"] = t1 - t0
        timings["modes_s"] = t2 - t1
    out = {
        "theta_deg": thetas.tolist(),
        "sigma_vv": (4.0 * math.pi * np.abs(F[0]) ** 2).tolist(),
        "sigma_hh": (4.0 * math.pi * np.abs(F[1]) ** 2).tolist(),
        "amp_vv": F[0].tolist(),
        "amp_hh": F[1].tolist(),
        "modes_used": modes_used,
        "n_unknowns": int(2 * Nn),
        "formulation": form,
        "linear_residual": max_res,
        "dF": np.array(dFs),
    }
    if keep_per_mode:
        out["per_mode"] = per_mode
    return out


def solve_bor_dielectric(points, freq_hz: float, thetas_deg, eps_r: complex, mu_r: complex = 1.0,
                         n_modes: Optional[int] = None, gauss_order: int = 4,
                         mode_tol: float = 1e-6, workers: int = 1) -> Dict:
    """Monostatic RCS of a closed homogeneous penetrable body by per-mode
    PMCHWT (bor_solver.py:1019-1095).  Unknowns J (2Nn) and M' = M / eta0
    (2Nn); with T the EFIE operator and P the rotated principal-value
    operator of each medium (exterior e, interior i):

        [ T_e + T_i             -eta0 (P_e + P_i)          ] [J ]   [ <W, E_inc>      ]
        [ eta0 (P_e + P_i)    T_e + (eta0/eta_i)^2 T_i     ] [M'] = [ eta0 <W, H_inc> ]

    and the far field radiates J and M in air."""
    thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
    if n_modes is None:
        n_modes = default_n_modes(points, freq_hz, thetas)
    m_max = int(n_modes)
    se = OracleSolver(points, freq_hz, gauss_order)
    si = OracleSolver(points, freq_hz, gauss_order, medium=(eps_r, mu_r))
    Nn = se.geo.Nn
    ones = np.ones(se.geo.P)
    for s in (se, si):
        s.prepare(m_max, efie=True, workers=workers, ibc_zs_pt=ones)
    eta_ratio2 = (ETA0 / si.eta) ** 2
    F = np.zeros((2, len(thetas)), dtype=np.complex128)

    def solve_am(am):
        dF = np.zeros_like(F)
        res = 0.0
        for m in ([0] if am == 0 else [am, -am]):
            T_e, T_i = se.assemble_efie(m, m_max), si.assemble_efie(m, m_max)
            P = ETA0 * (se.pmchwt_P(m, m_max) + si.pmchwt_P(m, m_max))
            A = np.block([[T_e + T_i, -P], [P, T_e + eta_ratio2 * T_i]])
            mask = np.tile(se.basis_mask(m), 2)
            A = A[np.ix_(mask, mask)]
            # <W, E_inc> and eta0 <W, H_inc> (bor_solver.py:647-657, 1068-1070)
            cols = [np.concatenate([se.rhs_efie(m, thetas, "VV"), -se.rhs_efie(m, thetas, "HH")], axis=1),
                    np.concatenate([se.rhs_efie(m, thetas, "HH"), se.rhs_efie(m, thetas, "VV")], axis=1)]
            B = np.stack(cols, axis=1).transpose(2, 0, 1).reshape(4 * Nn, 2 * len(thetas))[mask]
            X = np.linalg.solve(A, B)
            bn = float(np.linalg.norm(B))
            if bn > 0.0:
                res = max(res, float(np.linalg.norm(A @ X - B)) / bn)
            full = np.zeros((4 * Nn, X.shape[1]), dtype=np.complex128)
            full[mask] = X
            xs = full.T.reshape(len(thetas), 2, 4 * Nn)
            fth, _ = se.farfield(m, xs[:, 0, :2 * Nn], thetas, msol=ETA0 * xs[:, 0, 2 * Nn:])
            _, fph = se.farfield(m, xs[:, 1, :2 * Nn], thetas, msol=ETA0 * xs[:, 1, 2 * Nn:])
            dF[0] += fth
            dF[1] += fph
        return dF, res

    with ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        results = list(ex.map(solve_am, range(m_max + 1)))
    modes_used, quiet, max_res = 0, 0, 0.0
    for am, (dF, res) in enumerate(results):       # the reference's truncation (bor_solver.py:777-794)
        F += dF
        max_res = max(max_res, res)
        modes_used = am
        if float(np.max(np.abs(dF))) < mode_tol * max(float(np.max(np.abs(F))), 1e-30):
            quiet += 1
            if quiet >= 2:
                break
        else:
            quiet = 0
    return {
        "theta_deg": thetas.tolist(),
        "sigma_vv": (4.0 * math.pi * np.abs(F[0]) ** 2).tolist(),
        "sigma_hh": (4.0 * math.pi * np.abs(F[1]) ** 2).tolist(),
        "amp_vv": F[0].tolist(),
        "amp_hh": F[1].tolist(),
        "modes_used": modes_used,
        "n_unknowns": int(4 * Nn),
        "formulation": "pmchwt",
        "eps_r": complex(eps_r),
        "mu_r": complex(mu_r),
        "linear_residual": max_res,
    }


# ---------------------------------------------------------------------------
# two surfaces in one medium: cross operators and the coated PEC body
# ---------------------------------------------------------------------------

def _segment_distance(p0, p1, q0, q1) -> float:
    """Minimum distance of two non-crossing 2-D segments (bor_solver.py:1101-1112)."""
    def pt_seg(c, a, b):
        ab = b - a
        t = min(1.0, max(0.0, float(np.dot(c - a, ab) / max(np.dot(ab, ab), 1e-300))))
        return float(np.hypot(*(c - (a + t * ab))))
    return min(pt_seg(p0, q0, q1), pt_seg(p1, q0, q1), pt_seg(q0, p0, p1), pt_seg(q1, p0, p1))


class CrossOperators:
    """EFIE (T) and rotated principal-value (P) blocks between two different
    generatrices in one medium: test bases on sp, sources on sq
    (bor_solver.py:1115-1295).  Element pairs closer than near_factor times
    the longer element are integrated on a tensor Gauss grid of near_order
    points per side with the near kernels.  Surfaces that share an endpoint
    (coating junctions) are not restated here."""

    def __init__(self, sp: OracleSolver, sq: OracleSolver, near_factor: float = 2.0,
                 near_order: int = 12):
        if not np.isclose(complex(sp.k), complex(sq.k)):
            raise ValueError("Cross operators need both solvers in the same medium.")
        self.sp, self.sq, self.k, self.eta = sp, sq, sp.k, sp.eta
        self.near_order = near_order
        gp, gq = sp.geo, sq.geo
        diag = max(float(np.max(gp.nodes)) - float(np.min(gp.nodes)),
                   float(np.max(gq.nodes)) - float(np.min(gq.nodes)), 1e-9)
        touch = 1e-9 * diag
        self.near_pairs = []
        for e in range(gp.ne):
            pe = (gp.nodes[e], gp.nodes[e + 1])
            for f in range(gq.ne):
                qf = (gq.nodes[f], gq.nodes[f + 1])
                if any(float(np.hypot(*(a - b))) <= touch for a in pe for b in qf):
                    raise NotImplementedError("surfaces that share an endpoint (junctions)")
                d = _segment_distance(pe[0], pe[1], qf[0], qf[1])
                if d <= touch:
                    raise ValueError("Cross-operator surfaces cross or touch.")
                if d < near_factor * max(gp.lengths[e], gq.lengths[f]):
                    self.near_pairs.append((e, f))
        self._G = self._B = None
        self._near: Dict = {}

    def _tables(self, m_max: int):
        """Far kernels of every point pair by FFT over xi (bor_kernels.py:132-167,
        482-506), near pairs zeroed."""
        if self._G is not None:
            return self._G, self._B
        gp, gq, k = self.sp.geo, self.sq.geo, self.k
        rp, zp = gp.rho[:, None], gp.z[:, None]
        rq, zq = gq.rho[None, :], gq.z[None, :]
        osc = float(np.max(2.0 * abs(k) * np.sqrt(np.maximum(rp * rq, 0.0))))
        nx = int(2 ** math.ceil(math.log2(max(64, 4 * (m_max + 2), 6 * (osc + 4)))))
        xi = 2.0 * np.pi * np.arange(nx) / nx - np.pi
        d2 = (rp - rq) ** 2 + (zp - zq) ** 2
        R = np.maximum(np.sqrt(d2[..., None] + (4.0 * rp * rq)[..., None] * np.sin(0.5 * xi) ** 2),
                       1e-300)
        orders = np.arange(m_max + 2)
        G = np.fft.fft(np.exp(-1j * k * R) / (4.0 * np.pi * R), axis=-1)[..., :m_max + 2] \
            * (np.exp(1j * np.pi * orders) * (2.0 * np.pi / nx))
        nb = int(2 ** math.ceil(math.log2(max(128, 6 * (m_max + 2), 8 * (osc + 4)))))
        xib = 2.0 * np.pi * np.arange(nb) / nb - np.pi
        one = np.ones((gp.P, gq.P))
        a = [(v[:, None] * one).ravel() for v in (gp.rho, gp.z, gp.ptr, gp.ptz)]
        b = [(v[None, :] * one).ravel() for v in (gq.rho, gq.z, gq.ptr, gq.ptz)]
        ms = np.arange(-m_max, m_max + 1)
        bins = np.where(ms >= 0, ms, nb + ms)
        ph = np.exp(1j * np.pi * ms) * (2.0 * np.pi / nb)
        B = [(np.fft.fft(F, axis=-1)[:, bins] * ph).reshape(gp.P, gq.P, -1)
             for F in _ibc_bracket_grid(*a, *b, k, np.broadcast_to(xib, (a[0].size, nb)))]
        for (e, f) in self.near_pairs:
            sel = np.ix_(gp.elem == e, gq.elem == f)
            G[sel] = 0.0
            for Bi in B:
                Bi[sel] = 0.0
        self._G, self._B = G, B
        return G, B

    def _near_data(self, e: int, f: int, m_max: int):
        key = (e, f)
        if key in self._near:
            return self._near[key]
        x, w = np.polynomial.legendre.leggauss(self.near_order)
        u, w1 = 0.5 * (x + 1.0), 0.5 * w
        S, SP = np.meshgrid(u, u, indexing="ij")
        W = np.outer(w1, w1).ravel()
        gp, gq = self.sp.geo, self.sq.geo
        rp, zp, T0p, T1p, D0p, D1p, Lp = gp.points_on_element(e, S.ravel())
        rq, zq, T0q, T1q, D0q, D1q, Lq = gq.points_on_element(f, SP.ravel())
        Gm = near_G(rp, zp, rq, zq, self.k, m_max)
        Bn = near_ibc(rp, zp, np.full_like(rp, gp.trho[e]), np.full_like(rp, gp.tz[e]),
                      rq, zq, np.full_like(rq, gq.trho[f]), np.full_like(rq, gq.tz[f]), self.k, m_max)
        data = (W * Lp * Lq, rp, rq, np.vstack([T0p, T1p]), np.vstack([D0p, D1p]),
                np.vstack([T0q, T1q]), np.vstack([D0q, D1q]), Gm, Bn)
        self._near[key] = data
        return data

    def assemble_T(self, m: int, m_max: int) -> np.ndarray:
        """Cross EFIE operator [2Np, 2Nq], C = j k eta 2 pi of the medium
        (bor_solver.py:1221-1262, _pair_blocks :130-154)."""
        k, gp, gq = self.k, self.sp.geo, self.sq.geo
        G, _ = self._tables(m_max)
        am = abs(m)
        Gn = G[..., am]
        Gc = 0.5 * (G[..., abs(am - 1)] + G[..., am + 1])
        Gs = (G[..., abs(am - 1)] - G[..., am + 1]) / 2j
        if m < 0:
            Gs = -Gs
        rrw = (gp.rho * gp.w)[:, None] * (gq.rho * gq.w)[None, :]
        Ksc = gp.w[:, None] * gq.w[None, :] * Gn
        ztt = gp.BT @ (rrw * (np.outer(gp.ptr, gq.ptr) * Gc + np.outer(gp.ptz, gq.ptz) * Gn)) @ gq.BT.T \
            - (1.0 / k ** 2) * (gp.BD @ Ksc @ gq.BD.T)
        ztf = gp.BT @ (rrw * (gp.ptr[:, None] * Gs)) @ gq.BT.T - (1j * m / k ** 2) * (gp.BD @ Ksc @ gq.BT.T)
        zft = gp.BT @ (-rrw * (gq.ptr[None, :] * Gs)) @ gq.BT.T + (1j * m / k ** 2) * (gp.BT @ Ksc @ gq.BD.T)
        zff = gp.BT @ (rrw * Gc) @ gq.BT.T - (m ** 2 / k ** 2) * (gp.BT @ Ksc @ gq.BT.T)
        c = lambda A, kk, B: np.einsum("ip,p,jp->ij", A, kk, B)    # noqa: E731
        for (e, f) in self.near_pairs:
            w, rp, rq, Tp, Dp, Tq, Dq, Gt, _ = self._near_data(e, f, m_max)
            gn = Gt[:, am]
            gc = 0.5 * (Gt[:, abs(am - 1)] + Gt[:, am + 1])
            gs = (Gt[:, abs(am - 1)] - Gt[:, am + 1]) / 2j
            if m < 0:
                gs = -gs
            rr = rp * rq * w
            ksc = w * gn
            rs, cs = slice(e, e + 2), slice(f, f + 2)
            ztt[rs, cs] += c(Tp, rr * (gp.trho[e] * gq.trho[f] * gc + gp.tz[e] * gq.tz[f] * gn), Tq) \
                - (1.0 / k ** 2) * c(Dp, ksc, Dq)
            ztf[rs, cs] += c(Tp, rr * gp.trho[e] * gs, Tq) - (1j * m / k ** 2) * c(Dp, ksc, Tq)
            zft[rs, cs] += c(Tp, -rr * gq.trho[f] * gs, Tq) + (1j * m / k ** 2) * c(Tp, ksc, Dq)
            zff[rs, cs] += c(Tp, rr * gc, Tq) - (m ** 2 / k ** 2) * c(Tp, ksc, Tq)
        C = 1j * k * self.eta * 2.0 * np.pi
        return C * np.block([[ztt, ztf], [zft, zff]])

    def assemble_P(self, m: int, m_max: int) -> np.ndarray:
        """Cross rotated principal-value operator [2Np, 2Nq] (bor_solver.py:1264-1289)."""
        gp, gq = self.sp.geo, self.sq.geo
        _, Bt = self._tables(m_max)
        Wp = gp.BT * (gp.w * gp.rho)[None, :]
        Wq = gq.BT * (gq.w * gq.rho)[None, :]
        blocks = [2.0 * np.pi * Wp @ Bt[uv][..., m + m_max] @ Wq.T for uv in range(4)]
        for (e, f) in self.near_pairs:
            w, rp, rq, Tp, _, Tq, _, _, Bn = self._near_data(e, f, m_max)
            rr = rp * rq * w
            for uv in range(4):
                blocks[uv][e:e + 2, f:f + 2] += 2.0 * np.pi * np.einsum(
                    "ip,p,jp->ij", Tp, rr * Bn[uv][:, m + m_max], Tq)
        btt, btf, bft, bff = blocks
        return np.block([[-btf, btt], [-bff, bft]])


def solve_bor_coated_pec(points_outer, points_core, freq_hz: float, thetas_deg, eps_r: complex,
                         mu_r: complex = 1.0, n_modes: Optional[int] = None, gauss_order: int = 4,
                         mode_tol: float = 1e-6, near_factor: float = 2.0, near_order: int = 12,
                         workers: int = 1) -> Dict:
    """Monostatic RCS of a PEC core fully covered by a homogeneous coating
    (bor_solver.py:1298-1395).  Unknowns J_o, M'_o = M_o / eta0 on the outer
    interface and J_c on the core:

      [ T_e + T_L        -eta0 (P_e + P_L)          -T_L^oc      ] [J_o ]   [ V_E      ]
      [ eta0 (P_e + P_L)  T_e + (eta0/eta_L)^2 T_L  -eta0 P_L^oc ] [M'_o] = [ eta0 V_H ]
      [ T_L^co           -eta0 P_L^co               -T_L^cc      ] [J_c ]   [ 0        ]

    and only (J_o, M_o) radiate in air."""
    thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
    if n_modes is None:
        n_modes = default_n_modes(points_outer, freq_hz, thetas)
    m_max = int(n_modes)
    se = OracleSolver(points_outer, freq_hz, gauss_order)
    sLo = OracleSolver(points_outer, freq_hz, gauss_order, medium=(eps_r, mu_r))
    sLc = OracleSolver(points_core, freq_hz, gauss_order, medium=(eps_r, mu_r))
    Xoc = CrossOperators(sLo, sLc, near_factor, near_order)
    Xco = CrossOperators(sLc, sLo, near_factor, near_order)
    No, Nc = se.geo.Nn, sLc.geo.Nn
    ntot = 4 * No + 2 * Nc
    for s in (se, sLo):
        s.prepare(m_max, efie=True, workers=workers, ibc_zs_pt=np.ones(s.geo.P))
    sLc.prepare(m_max, efie=True, workers=workers)
    eta_ratio2 = (ETA0 / sLo.eta) ** 2
    iJ, iM, iC = slice(0, 2 * No), slice(2 * No, 4 * No), slice(4 * No, ntot)
    F = np.zeros((2, len(thetas)), dtype=np.complex128)

    def solve_am(am):
        dF = np.zeros_like(F)
        for m in ([0] if am == 0 else [am, -am]):
            P = ETA0 * (se.pmchwt_P(m, m_max) + sLo.pmchwt_P(m, m_max))
            T_e, T_L = se.assemble_efie(m, m_max), sLo.assemble_efie(m, m_max)
            A = np.zeros((ntot, ntot), dtype=np.complex128)
            A[iJ, iJ] = T_e + T_L
            A[iJ, iM] = -P
            A[iJ, iC] = -Xoc.assemble_T(m, m_max)
            A[iM, iJ] = P
            A[iM, iM] = T_e + eta_ratio2 * T_L
            A[iM, iC] = -ETA0 * Xoc.assemble_P(m, m_max)
            A[iC, iJ] = Xco.assemble_T(m, m_max)
            A[iC, iM] = -ETA0 * Xco.assemble_P(m, m_max)
            A[iC, iC] = -sLc.assemble_efie(m, m_max)
            mo = se.basis_mask(m)
            mask = np.concatenate([mo, mo, sLc.basis_mask(m)])
            A = A[np.ix_(mask, mask)]
            V = np.zeros((len(thetas), 2, ntot), dtype=np.complex128)
            V[:, 0, iJ], V[:, 0, iM] = se.rhs_efie(m, thetas, "VV"), -se.rhs_efie(m, thetas, "HH")
            V[:, 1, iJ], V[:, 1, iM] = se.rhs_efie(m, thetas, "HH"), se.rhs_efie(m, thetas, "VV")
            B = V.transpose(2, 0, 1).reshape(ntot, 2 * len(thetas))[mask]
            full = np.zeros((ntot, B.shape[1]), dtype=np.complex128)
            full[mask] = np.linalg.solve(A, B)
            xs = full.T.reshape(len(thetas), 2, ntot)
            fth, _ = se.farfield(m, xs[:, 0, iJ], thetas, msol=ETA0 * xs[:, 0, iM])
            _, fph = se.farfield(m, xs[:, 1, iJ], thetas, msol=ETA0 * xs[:, 1, iM])
            dF[0] += fth
            dF[1] += fph
        return dF

    with ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        results = list(ex.map(solve_am, range(m_max + 1)))
    modes_used, quiet = 0, 0
    for am, dF in enumerate(results):
        F += dF
        modes_used = am
        if float(np.max(np.abs(dF))) < mode_tol * max(float(np.max(np.abs(F))), 1e-30):
            quiet += 1
            if quiet >= 2:
                break
        else:
            quiet = 0
    return {"theta_deg": thetas.tolist(),
            "sigma_vv": (4.0 * math.pi * np.abs(F[0]) ** 2).tolist(),
            "sigma_hh": (4.0 * math.pi * np.abs(F[1]) ** 2).tolist(),
            "amp_vv": F[0].tolist(), "amp_hh": F[1].tolist(), "modes_used": modes_used,
            "n_unknowns": int(ntot), "formulation": "pmchwt-coated",
            "eps_r": complex(eps_r), "mu_r": complex(mu_r)}


def solve_multiregion(surfaces, regions, freq_hz: float, thetas_deg, n_modes: Optional[int] = None,
                      gauss_order: int = 4, mode_tol: float = 1e-6, near_factor: float = 2.0,
                      near_order: int = 12, workers: int = 1) -> Dict:
    """Multi-region PMCHWT for surfaces that meet no other surface off the
    axis (bor_solver.py:1805-2073 without junctions).  surfaces: [(points,
    is_conductor)]; regions: [{"medium": None | (eps, mu), "bounds":
    [(surface, sigma)], "exterior": bool}].  Unknowns per surface: J (2Nn)
    and, for interfaces, M' = M / eta0 (2Nn).  For every region r and ordered
    pair (i, j) of its bounding surfaces, with s = sigma_i sigma_j and the
    medium's operators: A[J_i, J_j] += s T, A[J_i, M_j] -= eta0 s P,
    A[M_i, J_j] += eta0 s P, A[M_i, M_j] += (eta0 / eta_r)^2 s T.  The
    exterior region's bounding surfaces carry the excitation and radiate."""
    thetas = np.atleast_1d(np.asarray(thetas_deg, dtype=float))
    is_cond = [bool(c) for (_, c) in surfaces]
    adj = [[] for _ in surfaces]
    for ri, reg in enumerate(regions):
        for (si, _) in reg["bounds"]:
            adj[si].append(ri)
    ext = next(ri for ri, r in enumerate(regions) if r.get("exterior"))
    solv = {(si, ri): OracleSolver(pts, freq_hz, gauss_order, medium=regions[ri]["medium"])
            for si, (pts, _) in enumerate(surfaces) for ri in adj[si]}
    for si in range(len(surfaces)):
        g = solv[(si, adj[si][0])].geo
        if not (g.on_axis(0) and g.on_axis(g.Nn - 1)):
            raise NotImplementedError("surfaces with off-axis ends (junctions)")
    X = {(ri, si, sj): CrossOperators(solv[(si, ri)], solv[(sj, ri)], near_factor, near_order)
         for ri, reg in enumerate(regions) for (si, _) in reg["bounds"] for (sj, _) in reg["bounds"]
         if si != sj}
    Nn = [solv[(si, adj[si][0])].geo.Nn for si in range(len(surfaces))]
    offJ, offM, n_full = [], [], 0
    for si in range(len(surfaces)):
        offJ.append(n_full)
        n_full += 2 * Nn[si]
        offM.append(None if is_cond[si] else n_full)
        n_full += 0 if is_cond[si] else 2 * Nn[si]
    if n_modes is None:
        k0 = 2.0 * math.pi * freq_hz / C0
        rho = max(float(np.max(np.asarray(p, float)[:, 0])) for p, _ in surfaces)
        n_modes = int(math.ceil(k0 * rho * max(float(np.max(np.abs(np.sin(np.radians(thetas))))), 0.05))) + 12
    m_max = int(n_modes)
    for (si, ri), s in solv.items():
        s.prepare(m_max, efie=True, workers=workers,
                  ibc_zs_pt=None if is_cond[si] else np.ones(s.geo.P))
    F = np.zeros((2, len(thetas)), dtype=np.complex128)

    def sl(off, si):
        return slice(off, off + 2 * Nn[si])

    def solve_am(am):
        dF = np.zeros_like(F)
        for m in ([0] if am == 0 else [am, -am]):
            A = np.zeros((n_full, n_full), dtype=np.complex128)
            for ri, reg in enumerate(regions):
                eta2 = (ETA0 / solv[(reg["bounds"][0][0], ri)].eta) ** 2
                for (si, gi) in reg["bounds"]:
                    for (sj, gj) in reg["bounds"]:
                        ss = gi * gj
                        if si == sj:
                            T = solv[(si, ri)].assemble_efie(m, m_max)
                            P = None if is_cond[si] else solv[(si, ri)].pmchwt_P(m, m_max)
                        else:
                            T = X[(ri, si, sj)].assemble_T(m, m_max)
                            P = X[(ri, si, sj)].assemble_P(m, m_max)
                        A[sl(offJ[si], si), sl(offJ[sj], sj)] += ss * T
                        if offM[sj] is not None:
                            A[sl(offJ[si], si), sl(offM[sj], sj)] += -ETA0 * ss * P
                        if offM[si] is not None:
                            A[sl(offM[si], si), sl(offJ[sj], sj)] += ETA0 * ss * P
                            if offM[sj] is not None:
                                A[sl(offM[si], si), sl(offM[sj], sj)] += eta2 * ss * T
            mask = np.zeros(n_full, dtype=bool)
            for si in range(len(surfaces)):
                bm = solv[(si, adj[si][0])].basis_mask(m)
                mask[sl(offJ[si], si)] = bm
                if offM[si] is not None:
                    mask[sl(offM[si], si)] = bm
            V = np.zeros((len(thetas), 2, n_full), dtype=np.complex128)
            for (si, _) in regions[ext]["bounds"]:
                s = solv[(si, ext)]
                vv, hh = s.rhs_efie(m, thetas, "VV"), s.rhs_efie(m, thetas, "HH")
                V[:, 0, sl(offJ[si], si)], V[:, 1, sl(offJ[si], si)] = vv, hh
                if offM[si] is not None:             # eta0 <W, H_inc>
                    V[:, 0, sl(offM[si], si)], V[:, 1, sl(offM[si], si)] = -hh, vv
            B = V.transpose(2, 0, 1).reshape(n_full, 2 * len(thetas))[mask]
            full = np.zeros((n_full, B.shape[1]), dtype=np.complex128)
            full[mask] = np.linalg.solve(A[np.ix_(mask, mask)], B)
            xs = full.T.reshape(len(thetas), 2, n_full)
            for (si, _) in regions[ext]["bounds"]:
                s = solv[(si, ext)]
                ms = [None if offM[si] is None else ETA0 * xs[:, p, sl(offM[si], si)] for p in (0, 1)]
                dF[0] += s.farfield(m, xs[:, 0, sl(offJ[si], si)], thetas, msol=ms[0])[0]
                dF[1] += s.farfield(m, xs[:, 1, sl(offJ[si], si)], thetas, msol=ms[1])[1]
        return dF

    with ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        results = list(ex.map(solve_am, range(m_max + 1)))
    modes_used, quiet = 0, 0
    for am, dF in enumerate(results):
        F += dF
        modes_used = am
        if float(np.max(np.abs(dF))) < mode_tol * max(float(np.max(np.abs(F))), 1e-30):
            quiet += 1
            if quiet >= 2:
                break
        else:
            quiet = 0
    return {"theta_deg": thetas.tolist(),
            "sigma_vv": (4.0 * math.pi * np.abs(F[0]) ** 2).tolist(),
            "sigma_hh": (4.0 * math.pi * np.abs(F[1]) ** 2).tolist(),
            "amp_vv": F[0].tolist(), "amp_hh": F[1].tolist(), "modes_used": modes_used,
            "n_unknowns": int(n_full)}


def solve_bor_coated2_pec(points_outer, points_mid, points_core, freq_hz: float, thetas_deg,
                          eps_inner: complex, mu_inner: complex, eps_outer: complex,
                          mu_outer: complex, **kw) -> Dict:
    """A PEC core under two full coating layers (bor_solver.py:2074-2098)."""
    return solve_multiregion(
        [(points_outer, False), (points_mid, False), (points_core, True)],
        [{"medium": None, "bounds": [(0, +1)], "exterior": True},
         {"medium": (eps_outer, mu_outer), "bounds": [(0, -1), (1, +1)]},
         {"medium": (eps_inner, mu_inner), "bounds": [(1, -1), (2, +1)]}],
        freq_hz, thetas_deg, **kw)
