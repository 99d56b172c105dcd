"""The oracle's C sampler restatement against the reference's own C sampler
(compiled from the reference source into oracle/_ref when available) and
against the NumPy formulas."""
import ctypes
import os

import numpy as np
import pytest

from conftest import REPO

dp = ctypes.POINTER(ctypes.c_double)


def _load(path, prefix):
    lib = ctypes.CDLL(path)
    g = getattr(lib, prefix + "sample_g")
    g.argtypes = [ctypes.c_int] * 3 + [dp] * 4 + [ctypes.c_double, dp, dp]
    h = getattr(lib, prefix + "sample_mfie")
    h.argtypes = [ctypes.c_int] * 3 + [dp] * 8 + [ctypes.c_double, dp, dp] + [dp] * 4
    return g, h


def _P(a):
    return a.ctypes.data_as(dp)


def _run(g, h):
    rng = np.random.default_rng(0)
    nr, npp, nx = 5, 9, 32
    a = [np.ascontiguousarray(rng.uniform(0, 1, nr)) for _ in range(4)]
    b = [np.ascontiguousarray(rng.uniform(0, 1, npp)) for _ in range(4)]
    xi = 2 * np.pi * np.arange(nx) / nx - np.pi
    s2 = np.ascontiguousarray(np.sin(0.5 * xi) ** 2)
    cx, sx = np.ascontiguousarray(np.cos(xi)), np.ascontiguousarray(np.sin(xi))
    o = np.empty((nr, npp, nx), np.complex128)
    g(nr, npp, nx, _P(a[0]), _P(a[1]), _P(b[0]), _P(b[1]), 7.5, _P(s2), _P(o))
    os_ = [np.empty((nr, npp, nx), np.complex128) for _ in range(4)]
    h(nr, npp, nx, *[_P(v) for v in a], *[_P(v) for v in b], 7.5, _P(cx), _P(sx), *[_P(v) for v in os_])
    return a, b, xi, o, os_


def test_sampler_matches_numpy(oracle):
    path = os.path.join(REPO, "oracle", "_build", "liboracle_sampler.so")
    g, h = _load(path, "oracle_")
    a, b, xi, o, os_ = _run(g, h)
    d2 = (a[0][:, None] - b[0][None, :]) ** 2 + (a[1][:, None] - b[1][None, :]) ** 2
    R = np.sqrt(d2[..., None] + 4 * (a[0][:, None] * b[0][None, :])[..., None] * np.sin(0.5 * xi) ** 2)
    ref = np.exp(-1j * 7.5 * R) / (4 * np.pi * R)
    assert np.max(np.abs(o - ref)) / np.max(np.abs(ref)) < 1e-14


def test_sampler_matches_reference_build(oracle):
    ref_path = os.path.join(REPO, "oracle", "_ref", "bor_stream_kernel.so")
    if not os.path.exists(ref_path):
        pytest.skip("reference sampler not built (reference tree absent)")
    mine = _run(*_load(os.path.join(REPO, "oracle", "_build", "liboracle_sampler.so"), "oracle_"))
    ref = _run(*_load(ref_path, ""))
    np.testing.assert_array_equal(mine[3], ref[3])
    for x, y in zip(mine[4], ref[4]):
        np.testing.assert_array_equal(x, y)
