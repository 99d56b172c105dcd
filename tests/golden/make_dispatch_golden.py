"""Generate tests/golden/dispatch.json, dispatch_grid.npz and tests/golden/grim/
by running the REFERENCE's dispatch layer (bor_dispatch, grim_io).

Run where the reference tree is mounted (its location from GHOST_REFERENCE_DIR):

    python tests/golden/make_dispatch_golden.py        # ~1 min

Two kinds of fixture:
  * host logic -- the reference's solve_monostatic_rcs_bor and
    solve_adaptive_frequency_sweep_bor with ``solve_bor`` replaced by the
    recording stand-in of tests/dispatch_stub.py: what reaches the solver
    (meshes bit for bit, frequencies, formulation) and the result rows;
    the exception type of each malformed input; bor_az_el_grid on the
    stand-in results; the .grim and dBke CSV files its exporters write.
  * end to end -- the reference's own FP64 solve (table_precision="double")
    of a small PEC sphere snapshot at two frequencies, VV and HH, and its
    radar-frame grid, for the GPU test of the same call.
"""

import copy
import json
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
REF = os.environ.get("GHOST_REFERENCE_DIR")
if not REF:
    raise SystemExit("set GHOST_REFERENCE_DIR to the reference tree")
sys.path.insert(0, REF)
sys.path.insert(0, TESTS)

import bor_dispatch as rd     # noqa: E402  (reference)
import grim_io as rg          # noqa: E402  (reference)
import dispatch_stub as stub  # noqa: E402


def main():
    out = {"cases": {}, "errors": {}}
    snaps = stub.snapshots()
    for name, snap, kw in stub.cases():
        rec = stub.Recorder()
        rd.solve_bor = rec
        rd.solve_bor_dielectric = rec.dielectric
        res = rd.solve_monostatic_rcs_bor(geometry_snapshot=snaps[snap], **kw)
        out["cases"][name] = {"calls": rec.calls, "result": res}
    for name, snap, kw in stub.bad_inputs():
        rd.solve_bor = stub.Recorder()
        rd.solve_bor_dielectric = rd.solve_bor.dielectric
        try:
            rd.solve_monostatic_rcs_bor(geometry_snapshot=snap, **kw)
            out["errors"][name] = None
        except Exception as exc:              # noqa: BLE001  (the type is the fixture)
            out["errors"][name] = type(exc).__name__
    rec = stub.Recorder()
    rd.solve_bor = rec
    out["adaptive"] = {
        "result": rd.solve_adaptive_frequency_sweep_bor(
            snaps["sphere_in"], 1.0, 3.0, [0.0, 45.0, 90.0], "VV", initial_points=5,
            max_refinements=3, db_threshold=3.0, max_total_points=12),
        "calls": [c["freq_hz"] for c in rec.calls]}

    # radar-frame grids of the stand-in VV / HH sweeps
    th = list(np.arange(0.0, 180.0001, 5.0))
    res = {}
    for pol in ("VV", "HH"):
        rd.solve_bor = stub.Recorder()
        res[pol] = rd.solve_monostatic_rcs_bor(snaps["sphere_in"], [1.0, 2.5], th, pol)
    grid = {}
    az, el = np.arange(-180.0, 180.1, 30.0), np.arange(-90.0, 90.1, 30.0)
    for tag, axis in (("horizontal", (0.0, 0.0)), ("tilted", (30.0, 20.0)),
                      ("vertical", (0.0, 90.0))):
        g = rd.bor_az_el_grid(res["VV"], res["HH"], az, el, *axis)
        grid[f"{tag}_theta"] = g["theta_map_deg"]
        for ch in ("VV", "HH", "VH"):
            grid[f"{tag}_{ch}"] = g["amp"][ch]
        if tag == "tilted":
            tilted = g
    out["grid_inputs"] = {"VV": res["VV"], "HH": res["HH"], "az": az.tolist(), "el": el.tolist()}

    # .grim files
    gdir = os.path.join(HERE, "grim")
    shutil.rmtree(gdir, ignore_errors=True)
    os.makedirs(gdir)
    rg.export_result_to_grim(res["VV"], os.path.join(gdir, "sphere_vv"), history="stand-in")
    rg.export_result_to_grim(out["cases"]["cone_sphere_efie_360"]["result"],
                             os.path.join(gdir, "cone_sphere_360.grim"),
                             preserve_raw_complex_amplitude=False, source_path="x.geo")
    bist = copy.deepcopy(res["HH"])
    bist["scattering_mode"] = "bistatic"
    for i, s in enumerate(bist["samples"]):
        s["theta_inc_deg"] = 0.0 if i % 2 else 22.5
    rg.export_result_to_grim(bist, os.path.join(gdir, "bistatic"), history="h")
    rg.save_bor_az_el_grim(tilted, os.path.join(gdir, "azel"), source_path="s", history="h")
    rg.export_result_to_dbke_csv(res["VV"], os.path.join(gdir, "sphere_vv"), source_path="a,b",
                                 history="h")

    # end to end: the reference's FP64 solve of a small sphere snapshot
    sph = {"segments": [stub.segment("s", stub.arc(0.1, 0.0, 0.0, 180.0, 16),
                                     ["2", "0", "0", "0", "0"])]}
    e2e_th = list(np.arange(0.0, 180.0001, 10.0))
    rd.solve_bor = __import__("bor_solver").solve_bor
    e2e = {}
    for pol in ("VV", "HH"):
        e2e[pol] = rd.solve_monostatic_rcs_bor(sph, [2.0, 3.0], e2e_th, pol,
                                               geometry_units="meters",
                                               table_precision="double", workers=8)
    g = rd.bor_az_el_grid(e2e["VV"], e2e["HH"], [0.0, 45.0, 90.0], [0.0, 30.0], 10.0, 5.0)
    for ch in ("VV", "HH", "VH"):
        grid[f"e2e_{ch}"] = g["amp"][ch]
    out["e2e"] = {"snapshot": sph, "thetas": e2e_th, "VV": e2e["VV"], "HH": e2e["HH"]}

    with open(os.path.join(HERE, "dispatch.json"), "w") as fh:
        json.dump(out, fh)
    np.savez(os.path.join(HERE, "dispatch_grid.npz"), **grid)
    print("errors:", out["errors"])
    print("adaptive:", out["adaptive"]["result"]["metadata"])


if __name__ == "__main__":
    main()
