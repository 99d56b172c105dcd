"""Error paths of the device code, driven safely from the host.

* Near fill: a workspace sized for a smaller tail order than some element pair
  needs.  The kernel skips those pairs (before touching the scratch), sets its
  status word and returns; the engine turns the status into RuntimeError.
* Tensor-core GEMM update: the pipeline waits are bounded.  With the limit at
  zero every pipeline wait gives up at once; the kernel still lets its copies
  in flight land (those drains keep the long limit), sets the status and
  returns without touching C, and the context stays usable: with the limit
  restored the same call gives the right product.
No fault, trap or endless wait is involved.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


def test_near_scratch_overflow_is_reported(pkg, torch):
    nat = pkg._native
    pts = pkg.bodies.cone_sphere_generatrix(0.5, 15.0, 40)
    prob = pkg.engine.BorGpuProblem(pts, 6.0 * 299792458.0 / (2 * math.pi), np.array([0.0, 90.0]), m_max=8)
    tails = prob.near.tails[:, 1]
    prob.n_tail_max = int(tails.min()) - 1          # too small for every pair
    band = torch.zeros((prob.m_max + 1, 4, prob.Nn, 5), dtype=torch.complex128, device="cuda")
    prob.fill_near(1.0 + 0.0j, nat.stream_handle(), band=band)
    torch.cuda.synchronize()
    with pytest.raises(RuntimeError, match="near kernel scratch too small"):
        prob.check_near_status()
    assert float(band.abs().max()) == 0.0            # every pair was skipped


def test_gemm_update_bounded_wait_gives_up_and_recovers(pkg, torch):
    nat = pkg._native
    lib = nat.load()
    rng = np.random.default_rng(3)
    batch, M, N, K = 2, 256, 64, 256                 # 16 K stages: the TMA warp must wait
    A = (rng.standard_normal((batch, M, K)) + 1j * rng.standard_normal((batch, M, K))).astype(np.complex64)
    B = (rng.standard_normal((batch, K, N)) + 1j * rng.standard_normal((batch, K, N))).astype(np.complex64)
    C0 = (rng.standard_normal((batch, M, N)) + 1j * rng.standard_normal((batch, M, N))).astype(np.complex64)
    dA, dB = torch.as_tensor(A, device="cuda"), torch.as_tensor(B, device="cuda")
    dC = torch.as_tensor(C0, device="cuda").clone()
    work = torch.empty(int(lib.ghost_bor_cgemm_tc_workspace(batch, M, N, K)), dtype=torch.uint8, device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    st = nat.stream_handle()
    args = (batch, M, N, K, nat.ptr(dA), K, M * K, nat.ptr(dB), N, K * N, nat.ptr(dC), N, M * N, nat.ptr(work))
    try:
        lib.ghost_bor_set_wait_limit(0)
        nat.call("ghost_bor_cgemm_tc", *args, nat.ptr(status), st)
        torch.cuda.synchronize()
    finally:
        lib.ghost_bor_set_wait_limit(-1)
    assert int(status.item()) == 1
    np.testing.assert_array_equal(dC.cpu().numpy(), C0)        # no tile was written
    nat.call("ghost_bor_cgemm_tc", *args, nat.ptr(status), st)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    want = C0.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    got = dC.cpu().numpy().astype(np.complex128)
    assert np.max(np.abs(got - want)) < 1e-4 * np.max(np.abs(want))
