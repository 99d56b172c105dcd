"""Host-side FP64 set-up of one body of revolution for the GPU kernels.

Everything here is O(N) or O(N * cells) NumPy work that fixes the discrete
problem exactly as the reference defines it:

* generatrix checks, element lengths and tangents (bor_kernels.py:38-82)
* 4-point Gauss data per element (bor_kernels.py:103-125), packed as the
  ``geo`` array the kernels read
* azimuth sample counts (bor_streaming.py:109-116) and the half-grid DCT /
  sin^2 tables equivalent to the reference's FFT over xi
* the graded near-cell quadrature (bor_solver.py:54-110), the per-pair tail
  order of the near kernel (bor_kernels.py:238-240), Gauss-Legendre tables
* the per-mode basis masks (bor_solver.py:611-622) as masked row indices
"""

from __future__ import annotations

import functools
import math
import os
import platform
from dataclasses import dataclass, field
from typing import Dict, List, Tuple

import numpy as np

C0 = 299_792_458.0
ETA0 = 376.730313668
AXIS_TOL = 1e-12
GEO_ROWS = 11      # rho, z, w, T0 w rho, T1 w rho, T0 w, T1 w, dRT0 w, dRT1 w, t_rho, t_z


_LEG_LO, _LEG_HI = 64, 1024          # the near tail orders
_LEG_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "leggauss_64_1024.npz")
_leg_table = None                    # (offsets, x, w) from _LEG_FILE, or False when absent / stale


def _leg_stamp() -> str:
    # the rules come from this machine's numpy / LAPACK: a table made elsewhere is stale
    return f"numpy {np.__version__} on {platform.machine()}"


def _leg_from_table(n: int):
    """Rule n from the table written at build time on this machine, or None."""
    global _leg_table
    if _leg_table is None:
        table = False
        try:
            with np.load(_LEG_FILE) as d:
                if str(d["stamp"]) == _leg_stamp():
                    table = (d["offsets"], d["x"], d["w"])
        except (OSError, KeyError, ValueError):
            pass
        _leg_table = table
    if not _leg_table:
        return None
    offs, x, w = _leg_table
    o = int(offs[n - _LEG_LO])
    return x[o:o + n].copy(), w[o:o + n].copy()


@functools.lru_cache(maxsize=None)
def _leggauss(n: int) -> Tuple[np.ndarray, np.ndarray]:
    """Gauss-Legendre nodes and weights on [-1, 1] (numpy's leggauss rule),
    cached: the near tail orders (up to 1024) repeat across element pairs,
    bodies and calls, and orders 64..1024 are also read from a table that the
    build writes with this same function (a fresh process then skips ~1-5 s
    of rule construction).  numpy finds the nodes as the eigenvalues of the
    symmetric tridiagonal Legendre companion matrix with a dense O(n^3)
    solver; the same eigenvalues come from the tridiagonal solver in O(n^2),
    followed by numpy's own Newton step, weights, symmetrisation and
    normalisation, which return the same nodes and weights as leggauss."""
    if _LEG_LO <= n <= _LEG_HI:
        r = _leg_from_table(n)
        if r is not None:
            x, w = r
            x.flags.writeable = False
            w.flags.writeable = False
            return x, w
    return _leggauss_compute(n)


def _leggauss_compute(n: int) -> Tuple[np.ndarray, np.ndarray]:
    L = np.polynomial.legendre
    try:
        from scipy.linalg import eigvalsh_tridiagonal
    except ImportError:               # pragma: no cover - scipy is in every image used
        eigvalsh_tridiagonal = None
    if n < 64 or eigvalsh_tridiagonal is None:
        x, w = L.leggauss(n)
    else:
        c = np.zeros(n + 1)
        c[-1] = 1.0
        m = L.legcompanion(c)
        x = eigvalsh_tridiagonal(np.diag(m).copy(), np.diag(m, 1).copy())
        dy = L.legval(x, c)
        df = L.legval(x, L.legder(c))
        x -= dy / df
        fm = L.legval(x, c[1:])
        fm /= np.abs(fm).max()
        df /= np.abs(df).max()
        w = 1.0 / (fm * df)
        w = (w + w[::-1]) / 2.0
        x = (x - x[::-1]) / 2.0
        w *= 2.0 / w.sum()
    x.flags.writeable = False
    w.flags.writeable = False
    return x, w


def _rules_for(ns):
    return [(n, _leggauss_compute(n)) for n in ns]


def write_leggauss_table(path: str = _LEG_FILE, workers: int = 1) -> str:
    """Compute every tail rule (orders 64..1024) with _leggauss_compute and
    store them in one file for _leggauss.  Serial by default (~15 s); with
    workers > 1 the orders are split over spawned processes, which only a
    caller whose main module is import-safe may ask for."""
    ns = list(range(_LEG_LO, _LEG_HI + 1))
    if workers > 1:
        import multiprocessing as mp
        from concurrent.futures import ProcessPoolExecutor
        chunks = [ns[i::workers] for i in range(workers)]
        with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
            rules = dict(r for part in ex.map(_rules_for, chunks) for r in part)
    else:
        rules = dict(_rules_for(ns))
    offsets = np.concatenate([[0], np.cumsum(ns[:-1])]).astype(np.int64)
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path[:-4] + ".tmp.npz"
    np.savez(tmp, offsets=offsets, x=np.concatenate([rules[n][0] for n in ns]),
             w=np.concatenate([rules[n][1] for n in ns]), stamp=_leg_stamp())
    os.replace(tmp, path)
    return path


def leggauss_table_ok(path: str = _LEG_FILE) -> bool:
    try:
        with np.load(path) as d:
            return str(d["stamp"]) == _leg_stamp() and len(d["offsets"]) == _LEG_HI - _LEG_LO + 1
    except (OSError, KeyError, ValueError):
        return False


class Generatrix:
    """Polyline generatrix in the (rho, z) half-plane, traversed from the +z
    axis end to the -z axis end (bor_kernels.py:38-82)."""

    def __init__(self, nodes):
        pts = np.array(nodes, dtype=float)
        if pts.ndim != 2 or pts.shape[1] != 2 or pts.shape[0] < 2:
            raise ValueError("Generatrix needs an (Nn, 2) array of (rho, z) nodes.")
        if np.any(pts[:, 0] < -1e-12):
            raise ValueError("Generatrix rho coordinates must be >= 0.")
        pts[:, 0] = np.maximum(pts[:, 0], 0.0)
        self.nodes = pts
        d = pts[1:] - pts[:-1]
        self.lengths = np.hypot(d[:, 0], d[:, 1])
        if np.any(self.lengths <= 0):
            raise ValueError("Generatrix has a zero-length element.")
        self.trho = d[:, 0] / self.lengths
        self.tz = d[:, 1] / self.lengths
        self.elem_n0 = np.arange(len(self.lengths))
        self.elem_n1 = self.elem_n0 + 1

    @property
    def n_elems(self) -> int:
        return len(self.lengths)

    @property
    def n_nodes(self) -> int:
        return len(self.nodes)

    def node_on_axis(self, i: int) -> bool:
        return self.nodes[i, 0] <= AXIS_TOL * max(1.0, float(np.max(self.nodes[:, 0])))


@dataclass
class GaussData:
    """Per-Gauss-point geometry (bor_kernels.py:84-101)."""
    elem: np.ndarray
    s: np.ndarray
    w: np.ndarray
    rho: np.ndarray
    z: np.ndarray
    trho: np.ndarray
    tz: np.ndarray
    T0: np.ndarray
    T1: np.ndarray
    dRT0: np.ndarray
    dRT1: np.ndarray


def gauss_on_generatrix(gen: Generatrix, order: int = 4) -> GaussData:
    xg, wg = _leggauss(order)
    s = 0.5 * (xg + 1.0)
    w = 0.5 * wg
    ne = gen.n_elems
    S = np.tile(s, ne)
    L = np.repeat(gen.lengths, order)
    r0 = gen.nodes[gen.elem_n0]
    r1 = gen.nodes[gen.elem_n1]
    drho = np.repeat(r1[:, 0] - r0[:, 0], order)
    rho = np.repeat(r0[:, 0], order) + S * drho
    z = np.repeat(r0[:, 1], order) + S * np.repeat(r1[:, 1] - r0[:, 1], order)
    return GaussData(
        elem=np.repeat(np.arange(ne), order), s=S, w=np.tile(w, ne) * L, rho=rho, z=z,
        trho=np.repeat(gen.trho, order), tz=np.repeat(gen.tz, order),
        T0=1.0 - S, T1=S, dRT0=(drho * (1.0 - S) - rho) / L, dRT1=(drho * S + rho) / L)


def pack_geo(g: GaussData) -> np.ndarray:
    """[GEO_ROWS][P] array read by the far, excitation and far-field kernels."""
    wr = g.w * g.rho
    return np.ascontiguousarray(np.stack([
        g.rho, g.z, g.w, g.T0 * wr, g.T1 * wr, g.T0 * g.w, g.T1 * g.w,
        g.dRT0 * g.w, g.dRT1 * g.w, g.trho, g.tz]))


def n_xi_efie(k: float, rho_max: float, m_max: int) -> int:
    """Azimuth samples of the Green's function sweep (bor_streaming.py:109-111)."""
    osc = 2.0 * abs(k) * rho_max
    return int(2 ** math.ceil(math.log2(max(64, 4 * (m_max + 2), 6 * (osc + 4)))))


def n_xi_bracket(k: float, rho_max: float, m_max: int) -> int:
    """Azimuth samples of the MFIE bracket sweep (bor_streaming.py:114-116)."""
    osc = 2.0 * abs(k) * rho_max
    return int(2 ** math.ceil(math.log2(max(128, 6 * (m_max + 2), 8 * (osc + 4)))))


def dct_tables(n_xi: int, n_orders: int, scale: float = 1.0) -> Tuple[np.ndarray, np.ndarray]:
    """Half-grid trapezoid/DCT-I weights equivalent to the reference's
    FFT over xi_l = -pi + 2 pi l / n_xi for an even integrand:

        G_n = (pi/h) [g_0 + (-1)^n g_h + 2 sum_{j=1}^{h-1} g_j cos(pi n j / h)],

    h = n_xi/2, g_j = g(pi j / h).  Returns dct [h+1, n_orders] (times
    ``scale``) and sin2 [h+1] = sin^2(pi j / n_xi)."""
    h = n_xi // 2
    j = np.arange(h + 1)
    n = np.arange(n_orders)
    c = np.full(h + 1, 2.0)
    c[0] = c[h] = 1.0
    # exact integer reduction of (n j) mod 2h keeps cos accurate for large n j
    nj = np.outer(j, n) % (2 * h)
    ang = np.pi * nj / h
    dct = (np.pi / h) * c[:, None] * np.cos(ang) * scale
    sin2 = np.sin(0.5 * np.pi * j / h) ** 2
    return np.ascontiguousarray(dct), np.ascontiguousarray(sin2)


def bracket_tables(n_xi: int, m_max: int) -> Tuple[np.ndarray, np.ndarray]:
    """Half-grid tables of the MFIE bracket transforms, m = 0..m_max.

    The reference takes the FFT of each of its four brackets over
    xi_l = -pi + 2 pi l / n_xi, keeps bins m (phase e^{j pi m} 2 pi / n_xi)
    and multiplies by the Galerkin 2 pi (bor_streaming.py:241-246, 378-385):
    K(m) = (4 pi^2 / n_xi) sum_l F(xi_l) e^{-j m xi_l}.  With
    s2 = sin^2(xi/2) and p = (1 + j k R) e^{-j k R} / R^3 every bracket is
    p (u + v s2) or sin(xi) p (u + v s2) with per-point-pair constants u, v,
    so three half-grid transforms of p cover all four (the 1/(4 pi) of the
    kernel is folded in):

        tab[0][j][m] = (pi/n) c_j cos(m xi_j)          c_j = 1, 2, ..., 2, 1
        tab[1][j][m] = (pi/n) c_j s2_j cos(m xi_j)
        tab[2][j][m] = (pi/n) 2 sin(xi_j) sin(m xi_j)  (zero at j = 0, h)

    xi_j = pi j / h, h = n_xi / 2.  Returns (tab [3, h+1, m_max+1], sin2 [h+1])."""
    h = n_xi // 2
    j = np.arange(h + 1)
    m = np.arange(m_max + 1)
    c = np.full(h + 1, 2.0)
    c[0] = c[h] = 1.0
    mj = np.outer(j, m) % (2 * h)
    ang = np.pi * mj / h
    xi = np.pi * j / h
    s2 = np.sin(0.5 * xi) ** 2
    sx = np.sin(np.pi * (j % (2 * h)) / h)
    sx[0] = sx[h] = 0.0
    f = np.pi / n_xi
    tab = np.empty((3, h + 1, m_max + 1))
    tab[0] = f * c[:, None] * np.cos(ang)
    tab[1] = tab[0] * s2[:, None]
    tab[2] = f * 2.0 * sx[:, None] * np.sin(ang)
    return np.ascontiguousarray(tab), np.ascontiguousarray(s2)


def element_mass(g: "GaussData", n_elem: int) -> np.ndarray:
    """Element contributions of the MFIE mass matrix 2 pi B_T diag(w rho) B_T^T
    (bor_solver.py:389-397): [n_elem, 4] = (a, b) in (0,0), (0,1), (1,0), (1,1)
    for nodes (e + a, e + b)."""
    wr = (g.w * g.rho).reshape(n_elem, -1)
    T = (g.T0.reshape(n_elem, -1), g.T1.reshape(n_elem, -1))
    out = np.empty((n_elem, 4))
    for a in range(2):
        for b in range(2):
            out[:, 2 * a + b] = 2.0 * np.pi * np.sum(T[a] * T[b] * wr, axis=1)
    return np.ascontiguousarray(out)


# ---------------------------------------------------------------------------
# graded near cells (bor_solver.py:54-110)
# ---------------------------------------------------------------------------

def graded_cells(kind: str, depth: int = 4) -> List[Tuple[float, float, float, float]]:
    """Cells (s0, s1, s'0, s'1) of [0,1]^2 refined toward the singular set:
    the diagonal (``diag``) or a shared corner (``cornerAB``: s = A, s' = B)."""
    cells: List[Tuple[float, float, float, float]] = []

    def singular(a0, a1, b0, b1):
        if kind == "diag":
            return not (a1 <= b0 or b1 <= a0)
        ca = 0.0 if kind[6] == "0" else 1.0
        cb = 0.0 if kind[7] == "0" else 1.0
        return a0 <= ca <= a1 and b0 <= cb <= b1

    def visit(a0, a1, b0, b1, level):
        if level >= depth or not singular(a0, a1, b0, b1):
            cells.append((a0, a1, b0, b1))
            return
        am, bm = 0.5 * (a0 + a1), 0.5 * (b0 + b1)
        visit(a0, am, b0, bm, level + 1)
        visit(a0, am, bm, b1, level + 1)
        visit(am, a1, b0, bm, level + 1)
        visit(am, a1, bm, b1, level + 1)

    visit(0.0, 1.0, 0.0, 1.0, 0)
    return cells


def cell_points(kind: str, gorder: int = 4) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Test points (order ``gorder``), source points (order ``gorder + 1``, so a
    test and a source point never coincide) and weights over the cells."""
    xs, ws = _leggauss(gorder)
    xq, wq = _leggauss(gorder + 1)
    us, vs = 0.5 * (xs + 1.0), 0.5 * ws
    uq, vq = 0.5 * (xq + 1.0), 0.5 * wq
    S, Q, W = [], [], []
    for (a0, a1, b0, b1) in graded_cells(kind):
        ha, hb = a1 - a0, b1 - b0
        ss, qq = np.meshgrid(a0 + us * ha, b0 + uq * hb, indexing="ij")
        S.append(ss.ravel())
        Q.append(qq.ravel())
        W.append(np.outer(vs * ha, vq * hb).ravel())
    return np.concatenate(S), np.concatenate(Q), np.concatenate(W)


_NEAR_KINDS = ("diag", "corner10", "corner01")


@dataclass
class NearTables:
    pairs: np.ndarray        # [n_pairs, 4] int32: e, f, cell offset, cell count
    tails: np.ndarray        # [n_pairs, 2] int32: tail offset, n_tail
    cells: np.ndarray        # [3, n_cells_total]
    core_gl: np.ndarray      # [2, 48]
    tail_gl: np.ndarray      # [4, n_tail_total]: u, w, and sin / cos(xi/2) of the node for s0 = 1/4
    n_tail: np.ndarray = field(default=None)


_NEAR_CELLS: Dict[int, tuple] = {}


def _near_cells(gorder: int = 4):
    """Cell points of the three near kinds, once per process: {kind: (offset,
    count, s, s')} and the concatenated [3, n_cells_total] table."""
    if gorder not in _NEAR_CELLS:
        kinds = {}
        off = 0
        blocks = []
        for kind in _NEAR_KINDS:
            s, sp_, w = cell_points(kind, gorder)
            kinds[kind] = (off, len(s), s, sp_)
            blocks.append(np.stack([s, sp_, w]))
            off += len(s)
        _NEAR_CELLS[gorder] = (kinds, np.ascontiguousarray(np.concatenate(blocks, axis=1)))
    return _NEAR_CELLS[gorder]


def near_tables(gen: Generatrix, k: float, m_max: int, core_order: int = 48) -> NearTables:
    """Element pairs |e - f| <= 1, their cell sets and the tail Gauss order
    n_tail = clip(ceil(4 (max|k| a / pi + m_max + 2)), 64, 1024) with
    a = sqrt(4 rho rho') over the pair's non-axis point pairs, bit-identical to
    the reference's choice (bor_kernels.py:199-204, 238-240).  The maximum is
    taken over 4 rho rho' before the (monotone, correctly rounded) square root
    and scaling, which gives the same value with one pass less per point."""
    ne = gen.n_elems
    kinds, cells = _near_cells()
    cells = cells.copy()
    kabs = abs(complex(k))
    x0 = gen.nodes[:-1, 0]
    dx = gen.nodes[1:, 0] - x0
    cols = []
    ntl = []
    for kind, df in (("diag", 0), ("corner10", 1), ("corner01", -1)):
        e = np.arange(max(0, -df), ne - max(0, df))
        f = e + df
        coff, cnt, s, sp_ = kinds[kind]
        mx = np.empty(len(e))
        # row blocks small enough to stay in cache
        for r0 in range(0, len(e), 64):
            eb, fb = e[r0:r0 + 64], f[r0:r0 + 64]
            rr4 = np.multiply.outer(dx[eb], s)
            rr4 += x0[eb][:, None]                  # rho on the test element
            rq = np.multiply.outer(dx[fb], sp_)
            rq += x0[fb][:, None]                   # rho' on the source element
            rr4 *= 4.0
            rr4 *= rq
            mx[r0:r0 + 64] = rr4.max(axis=1)
        on = mx > 1e-30                             # some point pair off the axis
        osc = kabs * np.sqrt(np.where(on, mx, 0.0)) / math.pi + (m_max + 2)
        nt = np.minimum(1024, np.maximum(64, np.ceil(4.0 * osc))).astype(np.int64)
        nt[~on] = 0
        cols.append(np.stack([e, f, np.full(len(e), coff), np.full(len(e), cnt)], axis=1))
        ntl.append(nt)
    pairs = np.concatenate(cols).astype(np.int32)
    ntails = np.concatenate(ntl)
    order = np.lexsort((pairs[:, 1], pairs[:, 0]))
    pairs = pairs[order]
    ntails = ntails[order]
    uniq = [int(n) for n in np.unique(ntails[ntails > 0])]
    tab_u, tab_w, offs = [], [], {}
    o = 0
    for n in uniq:
        x, wt = _leggauss(n)
        tab_u.append(0.5 * (x + 1.0))
        tab_w.append(0.5 * wt)
        offs[n] = o
        o += n
    if uniq:
        u = np.concatenate(tab_u)
        # the near kernels' tail nodes xi = xi0 + u (pi - xi0); for the common
        # core bound s0 = 1/4 (xi0 = 2 asin(1/4)) their half-angle sin / cos are
        # the same for every point pair, so they are tabulated here
        xi0 = 2.0 * math.asin(0.25)
        xi = xi0 + u * (math.pi - xi0)
        tail_gl = np.ascontiguousarray(np.stack([u, np.concatenate(tab_w), np.sin(0.5 * xi),
                                                 np.cos(0.5 * xi)]))
    else:
        tail_gl = np.zeros((4, 1))
    if uniq:
        u_arr = np.asarray(uniq, dtype=np.int64)
        o_arr = np.asarray([offs[n] for n in uniq], dtype=np.int64)
        pos = np.minimum(np.searchsorted(u_arr, ntails), len(uniq) - 1)
        toff = np.where(ntails > 0, o_arr[pos], 0)
    else:
        toff = np.zeros(len(ntails), dtype=np.int64)
    tails = np.stack([toff, ntails], axis=1).astype(np.int32)
    xc, wc = _leggauss(core_order)
    core_gl = np.ascontiguousarray(np.stack([0.5 * (xc + 1.0), 0.5 * wc]))
    return NearTables(pairs=np.ascontiguousarray(pairs), tails=np.ascontiguousarray(tails),
                      cells=cells, core_gl=core_gl, tail_gl=tail_gl, n_tail=ntails)


def basis_mask(gen: Generatrix, m: int) -> np.ndarray:
    """Active (J_t, J_phi) bases of mode m (bor_solver.py:611-622)."""
    Nn = gen.n_nodes
    t_act = np.ones(Nn, dtype=bool)
    f_act = np.ones(Nn, dtype=bool)
    for end in (0, Nn - 1):
        if gen.node_on_axis(end):
            t_act[end] = abs(m) == 1
            f_act[end] = False
        else:
            t_act[end] = False
            f_act[end] = True
    return np.concatenate([t_act, f_act])


def mask_rows(gen: Generatrix, m_max: int) -> np.ndarray:
    """[m_max+1, 4] int32 masked row indices per mode m >= 0 (-1 = unused)."""
    out = np.full((m_max + 1, 4), -1, dtype=np.int32)
    for m in range(m_max + 1):
        rows = np.flatnonzero(~basis_mask(gen, m))
        if len(rows) > 4:
            raise ValueError("basis mask removes more than four rows")
        out[m, :len(rows)] = rows
    return out


def default_n_modes(k: float, rho_max: float, thetas_deg) -> int:
    """bor_solver.py:845-847."""
    st = float(np.max(np.abs(np.sin(np.radians(np.atleast_1d(thetas_deg))))))
    return int(math.ceil(k * rho_max * max(st, 0.05))) + 12
