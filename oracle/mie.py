"""Mie-series backscatter of a PEC sphere -- TEST INFRASTRUCTURE ONLY.

Restates the reference's analytic oracle (mie_sphere.py:42-77 Riccati-Bessel
functions, :74-77 Wiscombe truncation, :96-101 PEC coefficients, :178-184
backscatter sum, :231-235 sigma_pec_sphere), e^{+jwt} convention.
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


def sigma_pec_sphere(radius_m: float, freq_hz: float) -> float:
    k = 2.0 * math.pi * freq_hz / C0
    x = k * radius_m
    nmax = max(6, int(math.ceil(x + 4.05 * x ** (1.0 / 3.0))) + 12)
    psi, dpsi = _psi(nmax, x)
    zeta, dzeta = _zeta(nmax, x)
    xi, dxi = psi - 1j * zeta, dpsi - 1j * dzeta
    a = -dpsi / dxi
    b = -psi / xi
    n = np.arange(1, nmax + 1)
    s = np.sum(((-1.0) ** n) * (2 * n + 1) * (a[1:] - b[1:]))
    lam = 2.0 * math.pi / k
    return float((lam ** 2 / (4.0 * math.pi)) * abs(s) ** 2)
