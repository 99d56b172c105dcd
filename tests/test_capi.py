"""The C-ABI library loads and exports every symbol include/ghost_bor.h declares
(no device calls)."""
import ctypes
import os
import re

import pytest

from conftest import REPO


def header_symbols():
    text = open(os.path.join(REPO, "include", "ghost_bor.h")).read()
    return sorted(set(re.findall(r"\b(ghost_bor_\w+)\s*\(", text)))


def test_header_lists_entry_points():
    syms = header_symbols()
    for s in ("ghost_bor_sample_g", "ghost_bor_far_efie", "ghost_bor_near_efie", "ghost_bor_rhs",
              "ghost_bor_getrf", "ghost_bor_getrs", "ghost_bor_residual", "ghost_bor_farfield"):
        assert s in syms


def test_library_exports_all(pkg):
    path = pkg.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    nat = pkg._native
    nat.load(path)
    assert set(nat.SIGNATURES) == set(header_symbols())
    assert lib.ghost_bor_version() >= 100


def test_bad_arguments_rejected(pkg):
    nat = pkg._native
    with pytest.raises(ValueError):
        nat.call("ghost_bor_getrf", nat.F32, 0, 10, 0, 10, 100, 0, 0, 0, 0)
    with pytest.raises(ValueError):
        nat.call("ghost_bor_far_efie", 7, 10, 3, 64, 1.0, 1.0, 0.0, 0, 0, 0, 0, 22, 484, 0)
