"""A .geo snapshot end to end on the GPU through bor_dispatch vs the reference.

The reference's solve_monostatic_rcs_bor solved a 0.1 m PEC sphere snapshot
(16 drawn primitives, meshed at 20 elements per wavelength) at 2 and 3 GHz,
VV and HH, in FP64 (tests/golden/make_dispatch_golden.py); its radar-frame
grid for a tilted axis is in dispatch_grid.npz.  Here the same call runs on the
GPU (both frequencies in one solve_bor_batch), in FP64 and in FP32 with FP64
refinement.  Named to run after the solver tests, so a failure here does not
hide their results.
"""
import importlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _amps(res):
    return np.array([complex(s["rcs_amp_real"], s["rcs_amp_imag"]) for s in res["samples"]])


@pytest.fixture(scope="module")
def e2e():
    with open(os.path.join(GOLDEN, "dispatch.json")) as fh:
        return json.load(fh)["e2e"]


@pytest.mark.parametrize("precision,tol", [("double", 1e-8), ("auto", 1e-4)])
def test_snapshot_sweep_and_grid_match_reference(pkg, e2e, precision, tol):
    D = importlib.import_module("20260722_ghost_gb300.bor_dispatch")
    res = {pol: D.solve_monostatic_rcs_bor(e2e["snapshot"], [2.0, 3.0], e2e["thetas"], pol,
                                           geometry_units="meters", table_precision=precision)
           for pol in ("VV", "HH")}
    for pol in ("VV", "HH"):
        got, want = _amps(res[pol]), _amps(e2e[pol])
        assert got.shape == want.shape
        assert np.max(np.abs(got - want)) / np.max(np.abs(want)) < tol
        db = [s["rcs_db"] for s in res[pol]["samples"]]
        db_ref = [s["rcs_db"] for s in e2e[pol]["samples"]]
        assert np.max(np.abs(np.subtract(db, db_ref))) < 0.01
        meta, meta_ref = res[pol]["metadata"], e2e[pol]["metadata"]
        assert meta["formulation"] == meta_ref["formulation"]
        for g, w in zip(meta["per_frequency"], meta_ref["per_frequency"]):
            assert g["n_unknowns"] == w["n_unknowns"]
            if precision == "double":
                assert g["modes_used"] == w["modes_used"]
    ref = np.load(os.path.join(GOLDEN, "dispatch_grid.npz"))
    g = D.bor_az_el_grid(res["VV"], res["HH"], [0.0, 45.0, 90.0], [0.0, 30.0], 10.0, 5.0)
    scale = max(np.max(np.abs(ref[f"e2e_{ch}"])) for ch in ("VV", "HH"))
    for ch in ("VV", "HH", "VH"):
        assert np.max(np.abs(g["amp"][ch] - ref[f"e2e_{ch}"])) < tol * scale


def test_rhs_h_mode_is_the_swapped_excitation(pkg):
    """BorPecSolver.rhs_h_mode (<W, H_inc>, bor_solver.py:647-657) against the
    reference's E excitations with the polarisations swapped, over eta0."""
    from conftest import load_golden
    bs = importlib.import_module("20260722_ghost_gb300.bor_solver")
    G = load_golden("sphere_n24")
    s = bs.BorPecSolver(G["points"], float(G["freq_hz"]))
    eta0 = 376.730313668
    for m in G["modes"]:
        m = int(m)
        for it, th in enumerate(G["thetas"][::3]):
            for pol, other, sign in (("VV", "HH", -1.0), ("HH", "VV", 1.0)):
                want = sign * G[f"Ve_{m}_{other}"][3 * it] / eta0
                got = s.rhs_h_mode(m, th, pol)
                assert np.max(np.abs(got - want)) <= 1e-12 * max(np.max(np.abs(want)), 1e-300)
