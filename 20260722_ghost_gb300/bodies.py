"""Generatrix builders for the benchmark bodies (host, FP64).

All generatrices run from the +z axis end to the -z axis end so the
left-of-travel normal points into the exterior, the convention of the
reference (bor_kernels.py:40-46).  Nodes are returned as an (Nn, 2) array of
(rho, z) in metres.

* ``sphere_generatrix``       -- the reference's canonical sphere
                                 (bor_solver.py:2179-2182): equal polar angle.
* ``cone_sphere_generatrix``  -- tangent cone-sphere: hemisphere of radius a,
                                 cone half-angle alpha, apex on +z at a/sin(alpha)
                                 from the sphere centre, tangency at polar angle
                                 90 deg - alpha; N equal-arc segments.
* ``random_body``             -- rho(s) = R0 sin(pi s)(1 + sum_k a_k sin(k pi s)),
                                 z(s) = L (1/2 - s), equal-arc in the generatrix.
* ``bspline_body``            -- clamped cubic B-spline radius profile on a 2 m
                                 axis with fixed zero-radius end points.
"""

from __future__ import annotations

import math
from typing import Dict, List, Sequence

import numpy as np

C0 = 299_792_458.0


def sphere_generatrix(a: float, n: int) -> np.ndarray:
    """North pole to south pole in equal polar-angle steps (bor_solver.py:2179-2182)."""
    th = np.linspace(0.0, math.pi, n + 1)
    return np.column_stack([a * np.sin(th), a * np.cos(th)])


def cylinder_generatrix(a: float, L: float, n_rad: int, n_len: int) -> np.ndarray:
    """Closed cylinder: top centre -> rim -> side -> bottom rim -> centre
    (bor_solver.py:2185-2190)."""
    top = np.column_stack([np.linspace(0.0, a, n_rad + 1), np.full(n_rad + 1, L / 2)])
    side = np.column_stack([np.full(n_len - 1, a), np.linspace(L / 2, -L / 2, n_len + 1)[1:-1]])
    bot = np.column_stack([np.linspace(a, 0.0, n_rad + 1), np.full(n_rad + 1, -L / 2)])
    return np.vstack([top, side, bot])


def cone_sphere_generatrix(a: float, half_angle_deg: float, n: int) -> np.ndarray:
    """Tangent cone-sphere with ``n`` equal-arc segments (see module doc)."""
    al = math.radians(half_angle_deg)
    z_apex = a / math.sin(al)
    th_t = 0.5 * math.pi - al
    tang = np.array([a * math.sin(th_t), a * math.cos(th_t)])
    apex = np.array([0.0, z_apex])
    L_cone = float(np.hypot(*(tang - apex)))
    L_arc = a * (math.pi - th_t)
    s = np.linspace(0.0, L_cone + L_arc, n + 1)
    pts = np.empty((n + 1, 2))
    on_cone = s <= L_cone
    t = s[on_cone] / L_cone
    pts[on_cone] = apex[None, :] + t[:, None] * (tang - apex)[None, :]
    th = th_t + (s[~on_cone] - L_cone) / a
    pts[~on_cone, 0] = a * np.sin(th)
    pts[~on_cone, 1] = a * np.cos(th)
    pts[0] = (0.0, z_apex)
    pts[-1] = (0.0, -a)
    return pts


def _equal_arc(curve, n: int, n_fine: int = 20001) -> np.ndarray:
    """Resample a parametric curve s -> (rho, z), s in [0, 1], at n equal arc steps."""
    s = np.linspace(0.0, 1.0, n_fine)
    xy = curve(s)
    seg = np.hypot(np.diff(xy[:, 0]), np.diff(xy[:, 1]))
    arc = np.concatenate([[0.0], np.cumsum(seg)])
    targets = np.linspace(0.0, arc[-1], n + 1)
    s_nodes = np.interp(targets, arc, s)
    pts = curve(s_nodes)
    pts[0, 0] = 0.0
    pts[-1, 0] = 0.0
    return pts


def random_body(rng: np.random.Generator, n: int):
    """One seeded random body of revolution; returns (points, arclen, params)."""
    L = rng.uniform(1.0, 4.0)
    R0 = rng.uniform(0.2, 0.8)
    ak = rng.uniform(-0.1, 0.1, size=6) / np.arange(1, 7)

    def curve(s):
        s = np.asarray(s, float)
        mod = 1.0 + sum(ak[i] * np.sin((i + 1) * np.pi * s) for i in range(6))
        return np.column_stack([R0 * np.sin(np.pi * s) * mod, L * (0.5 - s)])

    pts = _equal_arc(curve, n)
    arclen = float(np.sum(np.hypot(*np.diff(pts, axis=0).T)))
    return pts, arclen, {"L": L, "R0": R0, "a_k": ak.tolist()}


def random_bodies(n_bodies: int = 64, seed: int = 0) -> List[Dict]:
    """The seeded batch of random bodies: N ~ U{200..1600}, 12 segments per
    wavelength along the generatrix, |m| <= ceil(k rho_max) + 10."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_bodies):
        n = int(rng.integers(200, 1601))
        pts, arclen, params = random_body(rng, n)
        k = 2.0 * math.pi * n / (12.0 * arclen)
        m_max = int(math.ceil(k * float(np.max(pts[:, 0])))) + 10
        out.append({"points": pts, "n": n, "k": k, "freq_hz": k * C0 / (2.0 * math.pi),
                    "m_max": m_max, **params})
    return out


def bspline_basis(t: np.ndarray, n_ctrl: int, degree: int = 3) -> np.ndarray:
    """Clamped uniform B-spline basis [len(t), n_ctrl] (Cox-de Boor)."""
    n_inner = n_ctrl - degree - 1
    knots = np.concatenate([np.zeros(degree + 1),
                            np.arange(1, n_inner + 1) / (n_inner + 1),
                            np.ones(degree + 1)])
    t = np.clip(np.asarray(t, float), 0.0, 1.0)
    B = np.zeros((len(t), len(knots) - 1))
    for i in range(len(knots) - 1):
        B[:, i] = (knots[i] <= t) & (t < knots[i + 1])
    B[t >= 1.0, n_ctrl - 1] = 1.0
    for p in range(1, degree + 1):
        Bn = np.zeros((len(t), len(knots) - 1 - p))
        for i in range(len(knots) - 1 - p):
            d1 = knots[i + p] - knots[i]
            d2 = knots[i + p + 1] - knots[i + 1]
            a = (t - knots[i]) / d1 * B[:, i] if d1 > 0 else 0.0
            b = (knots[i + p + 1] - t) / d2 * B[:, i + 1] if d2 > 0 else 0.0
            Bn[:, i] = a + b
        B = Bn
    return B[:, :n_ctrl]


def bspline_body(radii: Sequence[float], n: int, half_length: float = 1.0):
    """Generatrix of a clamped cubic B-spline radius profile: control radii
    (0, r_1..r_J, 0) at equally spaced z from +half_length to -half_length,
    sampled at n + 1 nodes equally spaced in the spline parameter."""
    r = np.concatenate([[0.0], np.asarray(radii, float), [0.0]])
    zc = np.linspace(half_length, -half_length, len(r))
    t = np.linspace(0.0, 1.0, n + 1)
    B = bspline_basis(t, len(r))
    pts = np.column_stack([B @ r, B @ zc])
    pts[0, 0] = 0.0
    pts[-1, 0] = 0.0
    return pts, B
