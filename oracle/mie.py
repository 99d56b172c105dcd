"""Mie-series backscatter of a PEC sphere -- TEST INFRASTRUCTURE ONLY.

Restates the reference's analytic oracle (mie_sphere.py:42-77 Riccati-Bessel
functions, :74-77 Wiscombe truncation, :96-101 PEC coefficients, :104-121
Leontovich impedance coefficients, :178-184 backscatter sum, :231-242
sigma_pec_sphere / sigma_impedance_sphere), e^{+jwt} convention.
"""

import math

import numpy as np
from scipy import special as sp

C0 = 299_792_458.0


def _psi(nmax, x):
    n = np.arange(nmax + 1)
    jn = np.sqrt(np.pi / (2.0 * x)) * sp.jv(n + 0.5, x)
    jm1 = np.empty_like(jn)
    jm1[1:] = jn[:-1]
    jm1[0] = np.cos(x) / x
    return x * jn, x * jm1 - n * jn


def _zeta(nmax, x):
    n = np.arange(nmax + 1)
    yn = np.sqrt(np.pi / (2.0 * x)) * sp.yv(n + 0.5, x)
    ym1 = np.empty_like(yn)
    ym1[1:] = yn[:-1]
    ym1[0] = np.sin(x) / x
    return x * yn, x * ym1 - n * yn


ETA0 = 376.730313668


def _sphere_coefficients(x: float, g: complex):
    """Mie coefficients (A_n, B_n) of a sphere of size x whose surface obeys
    E_tan = Z_s n x H with g = j Z_s / eta0 (g = 0: PEC).  TM:
    dpsi + A dxi = g (psi + A xi); TE: psi + B xi = -g (dpsi + B dxi), the
    relative sign that gives zero backscatter at Z_s = eta0 (Weston)."""
    nmax = max(6, int(math.ceil(x + 4.05 * x ** (1.0 / 3.0))) + 12)
    psi, dpsi = _psi(nmax, x)
    zeta, dzeta = _zeta(nmax, x)
    xi, dxi = psi - 1j * zeta, dpsi - 1j * dzeta
    return -(dpsi - g * psi) / (dxi - g * xi), -(psi + g * dpsi) / (xi + g * dxi)


def _backscatter(k: float, a: np.ndarray, b: np.ndarray) -> float:
    n = np.arange(1, len(a))
    s = np.sum(((-1.0) ** n) * (2 * n + 1) * (a[1:] - b[1:]))
    lam = 2.0 * math.pi / k
    return float((lam ** 2 / (4.0 * math.pi)) * abs(s) ** 2)


def sigma_pec_sphere(radius_m: float, freq_hz: float) -> float:
    k = 2.0 * math.pi * freq_hz / C0
    return _backscatter(k, *_sphere_coefficients(k * radius_m, 0.0))


def sigma_impedance_sphere(radius_m: float, freq_hz: float, zs_ohm: complex) -> float:
    """Backscatter of a Leontovich (surface-impedance) sphere."""
    k = 2.0 * math.pi * freq_hz / C0
    return _backscatter(k, *_sphere_coefficients(k * radius_m, 1j * complex(zs_ohm) / ETA0))


def _causal_index(eps_r: complex, mu_r: complex) -> complex:
    """sqrt(eps_r mu_r) with Im <= 0 and Re >= 0."""
    m = np.sqrt(complex(eps_r) * complex(mu_r))
    if m.imag > 0.0:
        m = -m
    if m.real < 0.0:
        m = -m
    return m


def sigma_dielectric_sphere(radius_m: float, eps_r: complex, mu_r: complex, freq_hz: float) -> float:
    """Backscatter of a homogeneous (possibly lossy, magnetic) sphere: interior
    field C psi_n(m x); continuity of the tangential fields gives
    A_n = -(psi' psi_m - w psi_m' psi) / (xi' psi_m - w psi_m' xi) with
    w = m / eps_r (TM) or m / mu_r (TE)."""
    k = 2.0 * math.pi * freq_hz / C0
    x = k * radius_m
    m = _causal_index(eps_r, mu_r)
    X = max(x, abs(m) * x)
    nmax = max(6, int(math.ceil(X + 4.05 * X ** (1.0 / 3.0))) + 12)
    psi, dpsi = _psi(nmax, x)
    zeta, dzeta = _zeta(nmax, x)
    xi, dxi = psi - 1j * zeta, dpsi - 1j * dzeta
    psim, dpsim = _psi(nmax, m * x)
    wa, wb = m / complex(eps_r), m / complex(mu_r)
    a = -(dpsi * psim - wa * dpsim * psi) / (dxi * psim - wa * dpsim * xi)
    b = -(dpsi * psim - wb * dpsim * psi) / (dxi * psim - wb * dpsim * xi)
    return _backscatter(k, a, b)


def sigma_coated_pec_sphere(core_radius_m: float, outer_radius_m: float, eps_r: complex,
                            mu_r: complex, freq_hz: float) -> float:
    """Backscatter of a PEC sphere (radius b) inside one homogeneous layer
    (outer radius a): the layer field D psi_n(m k r) + E zeta_n(m k r) with
    E / D fixed by the PEC core (TM: U' = 0, TE: U = 0 at r = b), then the
    outer-interface continuity of the dielectric sphere."""
    if not (0.0 < core_radius_m < outer_radius_m):
        raise ValueError("Require 0 < core radius < outer radius.")
    k = 2.0 * math.pi * freq_hz / C0
    x = k * outer_radius_m
    m = _causal_index(eps_r, mu_r)
    X = max(x, abs(m) * x)
    nmax = max(6, int(math.ceil(X + 4.05 * X ** (1.0 / 3.0))) + 12)
    psi, dpsi = _psi(nmax, x)
    zeta, dzeta = _zeta(nmax, x)
    xi, dxi = psi - 1j * zeta, dpsi - 1j * dzeta
    pa, dpa = _psi(nmax, m * k * outer_radius_m)
    za, dza = _zeta(nmax, m * k * outer_radius_m)
    pb, dpb = _psi(nmax, m * k * core_radius_m)
    zb, dzb = _zeta(nmax, m * k * core_radius_m)
    out = []
    for ratio, w in ((dpb / dzb, m / complex(eps_r)), (pb / zb, m / complex(mu_r))):
        fa, dfa = pa - ratio * za, dpa - ratio * dza
        out.append(-(dpsi * fa - w * dfa * psi) / (dxi * fa - w * dfa * xi))
    return _backscatter(k, out[0], out[1])
