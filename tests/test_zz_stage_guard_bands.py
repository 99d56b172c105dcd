"""Out-of-bounds writes and non-finite outputs of every sweep stage (GPU).

compute-sanitizer is not available on the GPU pool, so each stage of one
CFIE sweep -- far and near fills (FP64 and FP32), excitation, composition,
FP32 and FP64 LU and solves, exact residual, tensor-core residual update,
far field -- writes into buffers placed inside larger allocations whose
64 KiB margins hold a sentinel (tests/guard_bands.py).  A stage passes when
no margin word changed and its outputs are finite.  The calls are the
engine's own, on contiguous buffers of the same shapes.  Named to run after
the parity tests, so a failure here does not hide their results.
"""
import math

import numpy as np
import pytest

from guard_bands import guarded

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(pkg):
    import torch
    eng, nat = pkg.engine, pkg._native
    pts = pkg.bodies.cone_sphere_generatrix(0.5, 15.0, 40)
    prob = eng.BorGpuProblem(pts, 20.0 * 299792458.0 / (2 * math.pi), np.linspace(0.0, 180.0, 7),
                             m_max=8, formulation="cfie")
    return torch, nat, prob


def _ok(torch, stage, checks, outs=()):
    torch.cuda.synchronize()
    for name, chk in checks.items():
        assert chk(), f"{stage}: a write landed outside {name}"
    for name, t in outs:
        assert bool(torch.isfinite(torch.view_as_real(t) if t.is_complex() else t).all()), \
            f"{stage}: {name} has non-finite entries"


def test_guard_bands_of_every_stage(env):
    torch, nat, p = env
    lib = nat.load()
    dev = p.device
    st = nat.stream_handle()
    Mb, n, nrhs, Nn = p.m_max + 1, p.n, p.nrhs, p.Nn
    c128, c64, i32, f64 = torch.complex128, torch.complex64, torch.int32, torch.float64

    # fills
    Zf, cZf = guarded((Mb, n, n), c128, dev)
    p.fill_operator_far(Zf, nat.F32, st)
    _ok(torch, "far fill (FP32)", {"Z_far": cZf}, [("Z_far", Zf)])
    band, cband = guarded((Mb, 4, Nn, 5), c128, dev)
    p.fill_operator_near(st, band=band, precision=nat.F32)
    _ok(torch, "near fill (band)", {"band": cband}, [("band", band)])
    Z64, cZ64 = guarded((Mb, n, n), c128, dev)
    p.fill_operator_far(Z64, nat.F64, st)
    p.fill_operator_near(st, Z=Z64)
    nat.call("ghost_bor_mask64", Mb, n, nat.ptr(p.d_masks), nat.ptr(Z64), n, Z64.stride(0), st)
    _ok(torch, "FP64 fill + mask", {"Z64": cZ64}, [("Z64", Z64)])
    p.check_near_status()

    # excitations
    B, cB = guarded((Mb, n, nrhs), c128, dev, zero=False)
    p.excitation(B, *p.excitation_coefs(), st)
    Ve, cVe = guarded((Mb, n, nrhs), c128, dev, zero=False)
    p.excitation(Ve, 1.0, 0.0, st)
    _ok(torch, "excitation", {"B": cB, "Ve": cVe}, [("B", B), ("Ve", Ve)])

    # FP32 operator, LU, solve
    A, cA = guarded((Mb, n, n), c64, dev, zero=False)
    nat.call("ghost_bor_compose", Mb, n, Nn, nat.ptr(Zf), n, Zf.stride(0), nat.ptr(band),
             nat.ptr(p.d_masks), nat.ptr(A), n, A.stride(0), st)
    Ac, cAc = guarded((Mb, n, n), c64, dev, zero=False)
    nat.call("ghost_bor_compose", Mb, n, Nn, nat.ptr(Zf), n, Zf.stride(0), nat.ptr(band),
             nat.ptr(p.d_masks), nat.ptr(Ac), n, Ac.stride(0), st)
    _ok(torch, "compose", {"A": cA, "Ac": cAc}, [("A", A)])
    ipiv, cpiv = guarded((Mb, n), i32, dev, zero=False)
    info, cinfo = guarded((Mb,), i32, dev, zero=False)
    lu_ws, clu = guarded((int(lib.ghost_bor_getrf_workspace(nat.F32, Mb, n)),), torch.uint8, dev)
    rs_ws, crs = guarded((int(lib.ghost_bor_getrs_workspace(nat.F32, Mb, n, nrhs)),), torch.uint8, dev)
    X32, cX32 = guarded((Mb, n, nrhs), c64, dev, zero=False)
    nat.call("ghost_bor_convert", 0, Mb, n, nrhs, nat.ptr(B), nrhs, B.stride(0), nat.ptr(X32),
             nrhs, X32.stride(0), st)
    nat.call("ghost_bor_getrf", nat.F32, Mb, n, nat.ptr(A), n, A.stride(0), nat.ptr(ipiv),
             nat.ptr(info), nat.ptr(lu_ws), st)
    nat.call("ghost_bor_getrs", nat.F32, Mb, n, nrhs, nat.ptr(A), n, A.stride(0), nat.ptr(ipiv),
             nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(rs_ws), st)
    X, cX = guarded((Mb, n, nrhs), c128, dev, zero=False)
    nat.call("ghost_bor_convert", 1, Mb, n, nrhs, nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(X),
             nrhs, X.stride(0), st)
    _ok(torch, "FP32 LU + solve", {"A": cA, "ipiv": cpiv, "info": cinfo, "lu_ws": clu, "rs_ws": crs,
                                   "X32": cX32, "X": cX}, [("A", A), ("X", X)])
    assert int(info.max()) == 0
    assert int(lu_ws[:4].view(torch.int32)[0]) == 0 and int(rs_ws[:4].view(torch.int32)[0]) == 0

    # exact residual and one tensor-core residual update
    R32, cR = guarded((Mb, n, nrhs), c64, dev, zero=False)
    norms, cn = guarded((Mb, 2), f64, dev, zero=False)
    ex_ws, cex = guarded((int(lib.ghost_bor_residual_exact_workspace(Mb, n, nrhs)),), torch.uint8, dev)
    nat.call("ghost_bor_residual_exact", Mb, n, nrhs, Nn, nat.ptr(Zf), n, Zf.stride(0), nat.ptr(band),
             nat.ptr(p.d_masks), nat.ptr(X32), nat.ptr(B), nrhs, B.stride(0), 0, nat.ptr(R32),
             nat.ptr(norms), nat.ptr(ex_ws), ex_ws.numel(), st)
    _ok(torch, "exact residual", {"R32": cR, "norms": cn, "ex_ws": cex}, [("R32", R32), ("norms", norms)])
    assert int(ex_ws[:4].view(torch.int32)[0]) == 0
    up_ws, cup = guarded((int(lib.ghost_bor_cgemm_tc_workspace(Mb, n, nrhs, n)),), torch.uint8, dev)
    status, cst = guarded((1,), i32, dev)
    D32, cD = guarded((Mb, n, nrhs), c64, dev, zero=False)
    D32.copy_(R32)
    nat.call("ghost_bor_cgemm_tc", Mb, n, nrhs, n, nat.ptr(Ac), n, Ac.stride(0), nat.ptr(D32), nrhs,
             D32.stride(0), nat.ptr(R32), nrhs, R32.stride(0), nat.ptr(up_ws), nat.ptr(status), st)
    _ok(torch, "residual update", {"R32": cR, "up_ws": cup, "status": cst, "D32": cD}, [("R32", R32)])
    assert int(status[0]) == 0

    # FP64 LU, solve, residual
    ipiv64, cp64 = guarded((Mb, n), i32, dev, zero=False)
    X64, cX64 = guarded((Mb, n, nrhs), c128, dev, zero=False)
    X64.copy_(B)
    Zc = Z64.clone()
    nat.call("ghost_bor_getrf", nat.F64, Mb, n, nat.ptr(Z64), n, Z64.stride(0), nat.ptr(ipiv64),
             nat.ptr(info), 0, st)
    nat.call("ghost_bor_getrs", nat.F64, Mb, n, nrhs, nat.ptr(Z64), n, Z64.stride(0), nat.ptr(ipiv64),
             nat.ptr(X64), nrhs, X64.stride(0), 0, st)
    nat.call("ghost_bor_residual64", Mb, n, nrhs, nat.ptr(Zc), n, Zc.stride(0), nat.ptr(X64),
             nat.ptr(B), nrhs, B.stride(0), 0, nat.ptr(norms), st)
    _ok(torch, "FP64 LU + solve + residual", {"Z64": cZ64, "ipiv64": cp64, "X64": cX64, "norms": cn},
        [("X64", X64), ("norms", norms)])
    assert int(info.max()) == 0

    # far field by reciprocity
    dF, cdF = guarded((Mb, nrhs), c128, dev)
    nat.call("ghost_bor_farfield", nat.F64, Mb, n, nrhs, Nn, p.k, nat.ptr(p.d_mode_w),
             nat.ptr(Ve), nrhs, Ve.stride(0), nat.ptr(X64), nrhs, X64.stride(0), nat.ptr(dF), st)
    _ok(torch, "far field", {"dF": cdF}, [("dF", dF)])
    # the FP32+IR first solve and the FP64 solve describe the same far field
    F32 = dF.sum(0)
    dF.zero_()
    nat.call("ghost_bor_farfield", nat.F64, Mb, n, nrhs, Nn, p.k, nat.ptr(p.d_mode_w),
             nat.ptr(Ve), nrhs, Ve.stride(0), nat.ptr(X), nrhs, X.stride(0), nat.ptr(dF), st)
    _ok(torch, "far field (FP32 solve)", {"dF": cdF}, [("dF", dF)])
    rel = float((dF.sum(0) - F32).abs().max() / F32.abs().max())
    assert rel < 1e-3, rel
