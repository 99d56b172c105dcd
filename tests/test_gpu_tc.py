"""Tensor-core (tcgen05, 3xTF32) complex GEMM update through the C ABI vs NumPy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# the last two cases have more tiles than SMs (each persistent CTA walks several
# tiles and reuses both TMEM accumulators) and many K stages
@pytest.mark.parametrize("batch,M,N,K", [(2, 200, 150, 64), (1, 128, 64, 8), (3, 77, 301, 37), (1, 300, 40, 200),
                                         (5, 1000, 700, 64), (2, 640, 900, 333)])
def test_cgemm_tc_matches_numpy(pkg, batch, M, N, K):
    import torch
    nat = pkg._native
    rng = np.random.default_rng(M + N + K)
    cplx = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)
    A, B, C = cplx(batch, M, K), cplx(batch, K, N), cplx(batch, M, N)
    want = C.astype(np.complex128) - A.astype(np.complex128) @ B.astype(np.complex128)
    dA, dB, dC = (torch.as_tensor(x, device="cuda") for x in (A, B, C))
    work = torch.empty(int(nat.load().ghost_bor_cgemm_tc_workspace(batch, M, N, K)), dtype=torch.uint8,
                       device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    nat.call("ghost_bor_cgemm_tc", batch, M, N, K, nat.ptr(dA), K, M * K, nat.ptr(dB), N, K * N,
             nat.ptr(dC), N, M * N, nat.ptr(work), nat.ptr(status), nat.stream_handle())
    got = dC.cpu().numpy()
    assert int(status.cpu()[0]) == 0
    scale = np.abs(A).max() * np.abs(B).max() * K
    err = np.abs(got - want).max() / scale
    assert err < 2e-6, err          # FP32-level: 3xTF32 split products, FP32 accumulation
