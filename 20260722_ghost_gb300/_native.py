"""ctypes binding of libghost_bor.so (the C ABI declared in include/ghost_bor.h).

The library is built in-tree by ``build.py``.  There is no CPU fallback: when
the library or a CUDA device is missing every entry point raises.
"""

from __future__ import annotations

import ctypes
import os
from typing import Optional

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libghost_bor.so")

OK, EINVAL, ECUDA, EUNSUPPORTED = 0, 1, 2, 3
F32, F64 = 0, 1

_vp = ctypes.c_void_p
_i = ctypes.c_int
_ll = ctypes.c_longlong
_d = ctypes.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "ghost_bor_version": (_i, []),
    "ghost_bor_last_error": (ctypes.c_char_p, []),
    "ghost_bor_launch_count": (_ll, []),
    "ghost_bor_sample_g": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _d, _vp, _vp, _vp]),
    "ghost_bor_sample_mfie": (_i, [_i, _i, _i] + [_vp] * 8 + [_d, _vp, _vp] + [_vp] * 4 + [_vp]),
    "ghost_bor_sample_ibc": (_i, [_i, _i, _i] + [_vp] * 8 + [_d, _vp, _vp] + [_vp] * 4 + [_vp]),
    "ghost_bor_far_efie": (_i, [_i, _i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_far_efie_masked": (_i, [_i, _i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _ll, _ll, _vp, _vp, _vp]),
    "ghost_bor_far_efie_tc_workspace": (_ll, [_i, _i, _i]),
    "ghost_bor_far_efie_tc_tables": (_i, [_i, _i, _vp, _vp, _vp, _ll, _vp]),
    "ghost_bor_far_efie_tc": (_i, [_i, _i, _i, _d, _d, _d, _vp, _vp, _ll, _vp, _ll, _ll, _vp]),
    "ghost_bor_far_efie_tc_masked": (_i, [_i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _ll, _vp, _ll, _ll, _vp]),
    "ghost_bor_set_near_grid": (_i, [_i]),
    "ghost_bor_near_workspace": (_ll, [_i]),
    "ghost_bor_near_efie": (_i, [_i, _i, _i, _d, _d, _d, _vp, _vp, _i, _vp, _vp, _vp, _i,
                                 _vp, _vp, _i, _vp, _vp, _ll, _ll, _i, _vp, _ll, _vp]),
    "ghost_bor_far_mfie": (_i, [_i, _i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_near_mfie_workspace": (_ll, [_i]),
    "ghost_bor_near_mfie": (_i, [_i, _i, _d, _d, _d, _vp, _vp, _vp, _i, _vp, _vp, _vp, _i,
                                 _vp, _vp, _i, _vp, _vp, _ll, _ll, _i, _vp, _ll, _vp]),
    "ghost_bor_far_ibc": (_i, [_i, _i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_near_ibc": (_i, [_i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _i,
                                _vp, _vp, _i, _vp, _vp, _ll, _ll, _i, _vp, _ll, _vp]),
    "ghost_bor_far_efie_ck": (_i, [_i, _i, _i, _d, _d, _d, _d, _vp, _vp, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_near_efie_ck": (_i, [_i, _i, _d, _d, _d, _d, _vp, _vp, _i, _vp, _vp, _vp, _i,
                                    _vp, _vp, _i, _vp, _vp, _ll, _ll, _i, _vp, _ll, _vp]),
    "ghost_bor_far_ibc_ck": (_i, [_i, _i, _i, _d, _d, _d, _d, _vp, _vp, _vp, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_near_ibc_ck": (_i, [_i, _i, _d, _d, _d, _d, _vp, _vp, _vp, _vp, _i, _vp, _vp, _vp, _i,
                                   _vp, _vp, _i, _vp, _vp, _ll, _ll, _i, _vp, _ll, _vp]),
    "ghost_bor_rhs_workspace": (_ll, [_i, _i, _i]),
    "ghost_bor_rhs": (_i, [_i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _ll, _ll, _vp, _vp]),
    "ghost_bor_rhs_weighted": (_i, [_i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _vp, _ll, _ll, _vp, _vp]),
    "ghost_bor_rhs_noalloc_capacity": (_ll, []),
    "ghost_bor_rhs_noalloc": (_i, [_i, _i, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_cgemm_tc_workspace": (_ll, [_i, _i, _i, _i]),
    "ghost_bor_set_wait_limit": (None, [_ll]),
    "ghost_bor_cgemm_tc": (_i, [_i, _i, _i, _i, _vp, _ll, _ll, _vp, _ll, _ll, _vp, _ll, _ll, _vp, _vp, _vp]),
    "ghost_bor_getrf_workspace": (_ll, [_i, _i, _i]),
    "ghost_bor_getrf": (_i, [_i, _i, _i, _vp, _ll, _ll, _vp, _vp, _vp, _vp]),
    "ghost_bor_getrs_workspace": (_ll, [_i, _i, _i, _i]),
    "ghost_bor_getrs": (_i, [_i, _i, _i, _i, _vp, _ll, _ll, _vp, _vp, _ll, _ll, _vp, _vp]),
    "ghost_bor_residual": (_i, [_i, _i, _i, _i, _vp, _ll, _ll, _vp, _vp, _vp, _vp, _ll, _ll,
                                _vp, _vp, _vp, _vp]),
    "ghost_bor_residual_x32": (_i, [_i, _i, _i, _i, _vp, _i, _ll, _ll, _vp, _vp, _vp, _vp, _ll, _ll,
                                    _vp, _vp, _vp, _vp]),
    "ghost_bor_split_words": (_i, [_i, _i, _i, _vp, _ll, _ll, _vp]),
    "ghost_bor_residual_exact_workspace": (_ll, [_i, _i, _i]),
    "ghost_bor_residual_exact": (_i, [_i, _i, _i, _i, _vp, _ll, _ll, _vp, _vp, _vp, _vp, _ll, _ll,
                                      _vp, _vp, _vp, _vp, _ll, _vp]),
    "ghost_bor_residual64": (_i, [_i, _i, _i, _vp, _ll, _ll, _vp, _vp, _ll, _ll, _vp, _vp, _vp]),
    "ghost_bor_farfield": (_i, [_i, _i, _i, _i, _i, _d, _vp, _vp, _ll, _ll, _vp, _ll, _ll, _vp, _vp]),
    "ghost_bor_compose": (_i, [_i, _i, _i, _vp, _ll, _ll, _vp, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_mask64": (_i, [_i, _i, _vp, _vp, _ll, _ll, _vp]),
    "ghost_bor_convert": (_i, [_i, _i, _i, _i, _vp, _ll, _ll, _vp, _ll, _ll, _vp]),
}

_LIB: Optional[ctypes.CDLL] = None


class NativeError(RuntimeError):
    pass


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load and bind the library (no device work)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise NativeError(
            f"{os.path.basename(path)} is not built; run "
            "`python -c \"import __graft_entry__ as g; g.build()\"` (nvcc, sm_103a) first")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def call(name: str, *args) -> int:
    """Invoke one C-ABI entry point and turn a non-zero status into an exception."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc == OK:
        return rc
    detail = lib.ghost_bor_last_error().decode(errors="replace") if rc == ECUDA else ""
    kind = {EINVAL: ValueError, EUNSUPPORTED: NotImplementedError}.get(rc, NativeError)
    raise kind(f"{name} failed with status {rc} {detail}".strip())


def launch_count() -> int:
    """Kernels launched by libghost_bor.so so far (counted at each launch)."""
    return int(load().ghost_bor_launch_count())


def ptr(t) -> int:
    """Device pointer of a torch tensor (or None -> NULL)."""
    return 0 if t is None else int(t.data_ptr())


def stream_handle(stream=None) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)
