"""The dispatch layer (bor_dispatch, grim_io) against the reference's, on CPU.

The reference's solve_monostatic_rcs_bor and solve_adaptive_frequency_sweep_bor
were run with the recording stand-in solver of dispatch_stub.py; the same
stand-in is patched into this package's bor_dispatch here, so every mesh the
solver receives must match bit for bit and every result row exactly.  The
radar-frame grid and the .grim files are compared with the reference's on the
same inputs (fixtures written by tests/golden/make_dispatch_golden.py).
"""
import importlib
import json
import os

import numpy as np
import pytest

import dispatch_stub as stub
from conftest import GOLDEN

D = importlib.import_module("20260722_ghost_gb300.bor_dispatch")
G = importlib.import_module("20260722_ghost_gb300.grim_io")


@pytest.fixture(scope="module")
def fx():
    with open(os.path.join(GOLDEN, "dispatch.json")) as fh:
        return json.load(fh)


@pytest.fixture
def rec(monkeypatch):
    r = stub.Recorder()
    monkeypatch.setattr(D, "solve_bor", r)
    monkeypatch.setattr(D, "solve_bor_batch", r.batch)
    monkeypatch.setattr(D, "solve_bor_dielectric", r.dielectric)
    return r


def _same_result(got, want, workers_given):
    for key, val in want.items():
        if key != "metadata":
            assert got[key] == val, key
    gm, wm = got["metadata"], want["metadata"]
    for key, val in wm.items():
        if key == "per_frequency":
            assert len(gm[key]) == len(val)
            for g, w in zip(gm[key], val):
                assert {k: g[k] for k in w} == w
        elif key != "workers" or workers_given:
            assert gm[key] == val, key


@pytest.mark.parametrize("name", [c[0] for c in stub.cases()])
def test_sweep_matches_reference(fx, rec, name):
    """Meshes handed to the solver, call arguments and result rows."""
    _, snap, kw = next(c for c in stub.cases() if c[0] == name)
    want = fx["cases"][name]
    got = D.solve_monostatic_rcs_bor(geometry_snapshot=stub.snapshots()[snap], **kw)
    assert len(rec.calls) == len(want["calls"])
    for g, w in zip(rec.calls, want["calls"]):
        assert g == w                                   # points bit for bit
    _same_result(got, want["result"], "workers" in kw)


@pytest.mark.parametrize("name", [c[0] for c in stub.bad_inputs()])
def test_bad_inputs_raise_like_reference(fx, rec, name):
    _, snap, kw = next(c for c in stub.bad_inputs() if c[0] == name)
    exc = {"ValueError": ValueError, "InterruptedError": InterruptedError,
           "FileNotFoundError": FileNotFoundError}[fx["errors"][name]]
    with pytest.raises(exc):
        D.solve_monostatic_rcs_bor(geometry_snapshot=snap, **kw)
    assert not rec.calls


def test_kinds_off_the_gpu_path_are_named(rec):
    """Valid coated bodies raise NotImplementedError; a conductor with an
    impedance flag goes to the solver (an IBC-EFIE when the flag has a model)."""
    arc = stub.arc(0.2, 0.0, 0.0, 180.0, 8)
    core = stub.arc(0.1, 0.0, 0.0, 180.0, 6)
    kw = dict(frequencies_ghz=[1.0], elevations_deg=[0.0], polarization="VV",
              geometry_units="meters")
    coated = {"segments": [stub.segment("o", arc, ["3", "0", "0", "1"]),
                           stub.segment("c", core, ["4", "0", "0", "1"])]}
    with pytest.raises(NotImplementedError, match="coated"):
        D.solve_monostatic_rcs_bor(coated, **kw)
    assert not rec.calls
    ibc = {"segments": [stub.segment("c", arc[:5], ["2", "0", "1"]),
                        stub.segment("c2", arc[4:], ["2"])],
           "ibcs": [["1", "constant", "120", "-30", "0", "0"]]}
    res = D.solve_monostatic_rcs_bor(ibc, **kw)
    assert res["metadata"]["formulation"] == "BoR-MoM IBC-EFIE (Leontovich)"
    (call,) = rec.calls
    zs = np.array([complex(*z) for z in call["zs"]])
    n_top = int(np.sum(np.asarray(call["points"])[:, 1] >= arc[4, 1] - 1e-12)) - 1
    assert call["formulation"] == "efie"
    assert np.all(zs[:n_top] == 120 - 30j) and np.all(zs[n_top:] == 0)


def test_one_mesh_per_frequency_goes_to_one_batch(monkeypatch):
    """Several frequencies reach the GPU as one solve_bor_batch call."""
    r = stub.Recorder()
    seen = []

    def batch(bodies, *a, **k):
        seen.append([b["freq_hz"] for b in bodies])
        return r.batch(bodies, *a, **k)

    monkeypatch.setattr(D, "solve_bor", None)
    monkeypatch.setattr(D, "solve_bor_batch", batch)
    D.solve_monostatic_rcs_bor(stub.snapshots()["sphere_in"], [1.0, 2.0, 3.0], [0.0, 45.0], "VV")
    assert seen == [[1e9, 2e9, 3e9]]


def test_progress_and_abort_between_frequencies(rec):
    import threading
    ev = threading.Event()
    log = []

    def progress(i, n, msg):
        log.append((i, n, msg))
        if i == 1:
            ev.set()
        raise RuntimeError("a failing callback must not stop the solve")

    with pytest.raises(InterruptedError):
        D.solve_monostatic_rcs_bor(stub.snapshots()["sphere_in"], [1.0, 2.0, 3.0], [0.0], "VV",
                                   progress_callback=progress, abort_event=ev)
    assert log == [(1, 3, "Solved 1 GHz")]
    assert len(rec.calls) == 1        # the abort is seen after the first frequency


def test_adaptive_sweep_matches_reference(fx, rec):
    want = fx["adaptive"]
    got = D.solve_adaptive_frequency_sweep_bor(
        stub.snapshots()["sphere_in"], 1.0, 3.0, [0.0, 45.0, 90.0], "VV", initial_points=5,
        max_refinements=3, db_threshold=3.0, max_total_points=12)
    assert [c["freq_hz"] for c in rec.calls] == want["calls"]
    assert got == want["result"]


@pytest.mark.parametrize("tag,axis", [("horizontal", (0.0, 0.0)), ("tilted", (30.0, 20.0)),
                                      ("vertical", (0.0, 90.0))])
def test_az_el_grid_matches_reference(fx, tag, axis):
    gi = fx["grid_inputs"]
    ref = np.load(os.path.join(GOLDEN, "dispatch_grid.npz"))
    g = D.bor_az_el_grid(gi["VV"], gi["HH"], gi["az"], gi["el"], *axis)
    assert np.max(np.abs(g["theta_map_deg"] - ref[f"{tag}_theta"])) < 1e-6
    scale = max(np.max(np.abs(ref[f"{tag}_{ch}"])) for ch in ("VV", "HH"))
    for ch in ("VV", "HH", "VH"):          # VH vanishes (to rounding) for a vertical axis
        want = ref[f"{tag}_{ch}"]
        assert g["amp"][ch].shape == want.shape
        assert np.max(np.abs(g["amp"][ch] - want)) <= 1e-12 * scale
        assert np.allclose(g["sigma"][ch], 4 * np.pi * np.abs(want) ** 2, rtol=1e-9,
                           atol=1e-20 * scale ** 2)
    assert g["frequencies_ghz"] == [1.0, 2.5]


def test_az_el_grid_rejects_swapped_or_mismatched(fx):
    gi = fx["grid_inputs"]
    with pytest.raises(ValueError):
        D.bor_az_el_grid(gi["HH"], gi["VV"], [0.0], [0.0])
    one = dict(gi["HH"], samples=[s for s in gi["HH"]["samples"] if s["frequency_ghz"] == 1.0])
    with pytest.raises(ValueError):
        D.bor_az_el_grid(gi["VV"], one, [0.0], [0.0])


def _grim_equal(a_path, b_path):
    a, b = np.load(a_path), np.load(b_path)
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        x, y = a[k], b[k]
        assert x.dtype == y.dtype, k
        assert x.shape == y.shape, k
        if x.dtype.kind == "f":
            assert np.array_equal(x, y, equal_nan=True), k
        else:
            assert np.array_equal(x, y), k


def test_grim_files_match_reference(fx, tmp_path):
    gi = fx["grid_inputs"]
    gdir = os.path.join(GOLDEN, "grim")
    written = []
    written += G.export_result_to_grim(gi["VV"], str(tmp_path / "sphere_vv"), history="stand-in")
    written += G.export_result_to_grim(fx["cases"]["cone_sphere_efie_360"]["result"],
                                       str(tmp_path / "cone_sphere_360.grim"),
                                       preserve_raw_complex_amplitude=False, source_path="x.geo")
    bist = json.loads(json.dumps(gi["HH"]))
    bist["scattering_mode"] = "bistatic"
    for i, s in enumerate(bist["samples"]):
        s["theta_inc_deg"] = 0.0 if i % 2 else 22.5
    written += G.export_result_to_grim(bist, str(tmp_path / "bistatic"), history="h")
    grid = D.bor_az_el_grid(gi["VV"], gi["HH"], gi["az"], gi["el"], 30.0, 20.0)
    written += G.save_bor_az_el_grim(grid, str(tmp_path / "azel"), source_path="s", history="h")
    written.append(G.export_result_to_dbke_csv(gi["VV"], str(tmp_path / "sphere_vv"), source_path="a,b",
                                               history="h"))
    assert sorted(os.path.basename(p) for p in written) == sorted(os.listdir(gdir))
    for p in written:
        name = os.path.basename(p)
        if name.endswith(".csv"):
            with open(p) as a, open(os.path.join(gdir, name)) as b:
                assert a.read() == b.read()
        elif name.startswith("azel"):
            # the grid itself agrees to 1e-12 (test above); the float32 files to rounding
            a, b = np.load(p), np.load(os.path.join(gdir, name))
            assert sorted(a.files) == sorted(b.files)
            live = b["rcs_power"] > 1e-12 * np.max(b["rcs_power"])   # phase is moot at zero
            for k in a.files:
                if k == "rcs_phase":
                    gap = np.angle(np.exp(1j * (a[k].astype(float) - b[k])))
                    assert np.max(np.abs(gap[live])) < 1e-5
                elif a[k].dtype.kind == "f":
                    assert np.allclose(a[k], b[k], rtol=1e-6, atol=1e-6 * np.max(np.abs(b[k])))
                else:
                    assert np.array_equal(a[k], b[k]), k
        else:
            _grim_equal(p, os.path.join(gdir, name))


def test_grim_duplicate_conflicts():
    row = {"frequency_ghz": 1.0, "theta_inc_deg": 10.0, "theta_scat_deg": 10.0,
           "rcs_linear": 2.0, "rcs_amp_real": 0.3, "rcs_amp_imag": 0.1}
    with pytest.raises(ValueError):
        G._cut_payload([row, dict(row, rcs_linear=3.0)], "VV", "", "", True, "dBsm", "sigma_3d")
    with pytest.raises(ValueError):
        G._cut_payload([row, dict(row, rcs_amp_imag=-0.1)], "VV", "", "", True, "dBsm",
                       "sigma_3d")
    p = G._cut_payload([row, dict(row)], "VV", "", "", True, "dBsm", "sigma_3d")
    assert p["rcs_power"].shape == (1, 1, 1, 1)
    with pytest.raises(ValueError):
        G.export_result_to_grim({"samples": []}, "unused")
