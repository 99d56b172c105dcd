"""The allocation-free excitation entry point (ghost_bor_rhs_noalloc).

Callers that cannot allocate device memory during a solve -- a service that
reserves all GPU memory for its own arena, or a thread that must not call
cudaMalloc/cudaFree because those calls can synchronise the device -- get the
excitation from a workspace that lives in a static device array inside the
library.  This file checks, through the C ABI, that two calls in a row give the
same excitation as ghost_bor_rhs with a caller workspace, including a problem
that needs several angle blocks, and that oversized problems are rejected.
It is named to be collected last (after every test_zz_* file) so a failure
here does not hide other results.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def _problem(pkg, N, M, n_theta):
    eng = pkg.engine
    pts = pkg.bodies.cone_sphere_generatrix(0.5, 15.0, N)
    k = 30.0
    return eng.BorGpuProblem(pts, k * 299_792_458.0 / (2 * math.pi),
                             np.linspace(0.0, 180.0, n_theta), m_max=M)


@pytest.mark.parametrize("N,M,n_theta", [(60, 8, 37), (600, 40, 181)])
def test_noalloc_matches_workspace_entry_point(pkg, torch, N, M, n_theta):
    nat = pkg._native
    p = _problem(pkg, N, M, n_theta)
    st = nat.stream_handle()
    shape = (p.m_max + 1, p.n, p.nrhs)
    ref = torch.empty(shape, dtype=torch.complex128, device="cuda")
    work = p.excitation(ref, 1.0, 0.5, st)
    per_angle = 4 * p.N * ((p.m_max + 2) * 8 + 16)
    blocks = math.ceil(p.T / ((nat.load().ghost_bor_rhs_noalloc_capacity() - 256) // per_angle))
    if N == 600:
        assert blocks > 1          # the large case exercises several angle blocks
    for _ in range(2):             # two calls in a row share the static workspace
        out = torch.full(shape, complex(np.nan, np.nan), dtype=torch.complex128, device="cuda")
        nat.call("ghost_bor_rhs_noalloc", p.N, p.m_max, p.T, p.k, 1.0, 0.5, nat.ptr(p.d_geo),
                 nat.ptr(p.d_thetas), nat.ptr(p.d_masks), nat.ptr(out), out.shape[-1], out.stride(0), st)
        torch.cuda.synchronize()
        a, b = out.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(b))
    del work


def test_noalloc_rejects_oversized(pkg, torch):
    nat = pkg._native
    cap = nat.load().ghost_bor_rhs_noalloc_capacity()
    n_elem, m_max = 5000, 500          # one angle needs 4*5000*502*8 bytes > 64 MiB
    assert 4 * n_elem * ((m_max + 2) * 8 + 16) > cap
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    masks = torch.full((m_max + 1, 4), -1, dtype=torch.int32, device="cuda")
    with pytest.raises(ValueError):
        nat.call("ghost_bor_rhs_noalloc", n_elem, m_max, 1, 1.0, 1.0, 0.0, nat.ptr(dummy),
                 nat.ptr(dummy), nat.ptr(masks), nat.ptr(dummy), 2, 2 * 2 * (n_elem + 1), 0)
