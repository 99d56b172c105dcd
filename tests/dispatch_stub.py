"""A deterministic stand-in for ``solve_bor`` used to test the dispatch layer.

The dispatch layer (snapshot checks, meshing, frequency loop, sample rows,
aspect mirroring, adaptive refinement, radar-frame grid, .grim export) is host
code; its parity with the reference is checked by running the reference's
``bor_dispatch`` and this package's ``bor_dispatch`` with the same stand-in
solver, which records every call and returns amplitudes that are a smooth,
exactly reproducible function of the mesh, frequency and aspect.  The fixture
generator (tests/golden/make_dispatch_golden.py) and the tests import this
module, so both sides see identical solver outputs.
"""
import copy
import math
import os
import threading

import numpy as np

C0 = 299_792_458.0
# mat.<flag> table files of the impedance cases
MATERIALS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "materials")


class Recorder:
    """Callable stand-in for solve_bor; ``calls`` logs what it was given."""

    def __init__(self):
        self.calls = []

    def __call__(self, points, freq_hz, thetas_deg, formulation="efie", cfie_alpha=0.5,
                 zs=None, n_modes=None, mode_tol=1e-6, table_precision="auto", **_kw):
        pts = np.asarray(points, dtype=float)
        th = np.radians(np.asarray(thetas_deg, dtype=float))
        zrec = None if zs is None else [[float(z.real), float(z.imag)]
                                        for z in np.atleast_1d(np.asarray(zs, dtype=complex))]
        self.calls.append({"points": pts.tolist(), "freq_hz": float(freq_hz),
                           "thetas": np.degrees(th).tolist(), "formulation": formulation,
                           "cfie_alpha": float(cfie_alpha), "n_modes": n_modes,
                           "mode_tol": float(mode_tol), "table_precision": table_precision,
                           "zs": zrec})
        k = 2.0 * math.pi * float(freq_hz) / C0
        n = len(pts)
        sig = float(np.sum(pts[:, 0]) - 0.5 * np.sum(pts[:, 1]))
        ph = 0.01 * k * sig + 3.0 * th
        mag_v = (1.0 + 0.9 * np.cos(2.0 * th + 0.31 * k)) * n / 50.0
        mag_h = (1.2 + 0.7 * np.sin(3.0 * th - 0.17 * k)) * n / 50.0
        amp_vv = mag_v * np.exp(1j * ph)
        amp_hh = mag_h * np.exp(-0.7j * ph)
        amp_vv[np.abs(np.degrees(th) - 90.0) < 1e-12] = 0.0      # a null: the 1e-30 floor
        warnings = ["stand-in warning A"] + (["stand-in warning B"] if freq_hz > 2e9 else [])
        return {
            "theta_deg": np.degrees(th).tolist(),
            "sigma_vv": (4.0 * math.pi * np.abs(amp_vv) ** 2).tolist(),
            "sigma_hh": (4.0 * math.pi * np.abs(amp_hh) ** 2).tolist(),
            "amp_vv": amp_vv.tolist(), "amp_hh": amp_hh.tolist(),
            "modes_used": 5 + n % 7, "n_unknowns": 2 * n - 4,
            "linear_residual": 1e-13 * n, "warnings": warnings,
        }

    def dielectric(self, points, freq_hz, thetas_deg, eps_r, mu_r=1.0, n_modes=None, mode_tol=1e-6,
                   **_kw):
        """Stand-in for solve_bor_dielectric: logged with the medium, the same
        smooth amplitude model scaled by the medium."""
        out = self(points, freq_hz, thetas_deg, formulation="pmchwt", n_modes=n_modes, mode_tol=mode_tol)
        call = self.calls[-1]
        call["eps_r"] = [complex(eps_r).real, complex(eps_r).imag]
        call["mu_r"] = [complex(mu_r).real, complex(mu_r).imag]
        g = abs(complex(eps_r) * complex(mu_r)) ** 0.25
        for key in ("amp_vv", "amp_hh"):
            out[key] = [a * g for a in out[key]]
        for key, amp in (("sigma_vv", "amp_vv"), ("sigma_hh", "amp_hh")):
            out[key] = [4.0 * math.pi * abs(a) ** 2 for a in out[amp]]
        out["n_unknowns"] = 2 * out["n_unknowns"]
        return out

    def batch(self, bodies, thetas_deg, formulation="efie", cfie_alpha=0.5, mode_tol=1e-6,
              table_precision="auto", progress=None):
        """Stand-in for solve_bor_batch: one call per body, in order."""
        out = []
        for i, b in enumerate(bodies):
            out.append(self(b["points"], b["freq_hz"], thetas_deg, formulation=formulation,
                            cfie_alpha=cfie_alpha, n_modes=b.get("n_modes"),
                            mode_tol=mode_tol, table_precision=table_precision))
            if progress is not None:
                progress(i + 1, len(bodies))
        return out


def arc(radius, z0, t0_deg, t1_deg, n):
    """Polyline (rho, z) on a circle about (0, z0) from polar angle t0 to t1."""
    t = np.radians(np.linspace(t0_deg, t1_deg, n + 1))
    return np.stack([radius * np.sin(t), z0 + radius * np.cos(t)], axis=1)


def segment(name, pts, props):
    pairs = [{"x1": float(a[0]), "y1": float(a[1]), "x2": float(b[0]), "y2": float(b[1])}
             for a, b in zip(pts[:-1], pts[1:])]
    seg = {"name": name, "point_pairs": pairs}
    if props is not None:
        seg["properties"] = props
    return seg


def snapshots():
    """The snapshots both sides are run on (all valid PEC bodies)."""
    sphere = {"segments": [segment("sphere", arc(6.0, 0.0, 0.0, 180.0, 12),
                                   ["2", "0", "0", "0", "0"])]}
    # 15-degree cone-sphere, hemisphere radius 0.2 m, drawn as three segments listed
    # out of order, with fixed-count and per-wavelength densities
    a, half = 0.2, math.radians(15.0)
    apex = a / math.sin(half)
    tang = np.array([a * math.cos(half), a * math.sin(half)])
    cone = np.stack([np.linspace(0.0, tang[0], 4), np.linspace(apex, tang[1], 4)], axis=1)
    cone[0] = (0.0, apex)
    cap1 = arc(a, 0.0, 75.0, 130.0, 5)
    cap1[0] = tang
    cap2 = arc(a, 0.0, 130.0, 180.0, 4)
    cap2[0] = cap1[-1]
    cone_sphere = {"segments": [segment("cap-b", cap2, ["2", "-12", "mat.0", "0", "0"]),
                                segment("flank", cone, ["2", "3", "", "", ""]),
                                segment("cap-a", cap1, ["2.0", "5"])]}
    # an ogive-like body with missing and malformed properties, drawn in inches
    ogive = {"segments": [segment("nose", arc(10.0, -4.0, 0.0, 60.0, 6), None),
                          segment("tail", np.vstack([arc(10.0, -4.0, 60.0, 90.0, 3),
                                                     [[0.0, -10.0]]]),
                                  ["2", "junk"])]}
    ogive["segments"][1]["point_pairs"][0]["x1"] = ogive["segments"][0]["point_pairs"][-1]["x2"]
    ogive["segments"][1]["point_pairs"][0]["y1"] = ogive["segments"][0]["point_pairs"][-1]["y2"]
    # impedance flags: the cone-sphere with a constant Z_s on the flank, a
    # linear taper on one cap and a frequency table (tests/golden/materials/
    # mat.51) on the other; unused medium rows are parsed too
    cone_ibc = copy.deepcopy(cone_sphere)
    cone_ibc["segments"][0]["properties"] = ["2", "-12", "51", "0", "0"]
    cone_ibc["segments"][1]["properties"] = ["2", "3", "1", "", ""]
    cone_ibc["segments"][2]["properties"] = ["2.0", "5", "mat.2"]
    cone_ibc["ibcs"] = [["1", "constant", "50", "-20", "0", "0"],
                        ["mat.2", "Linear", "0", "0", "100", "-50"], ["51"], [], ["0", "x"]]
    cone_ibc["dielectrics"] = [["3", "4.0", "-0.1", "1", "0"], ["4", "0", "0"], ["5"]]
    # a sphere in two segments: a raised-cosine taper from PEC and a geometric
    # taper, in inches
    top, bottom = arc(6.0, 0.0, 0.0, 100.0, 7), arc(6.0, 0.0, 100.0, 180.0, 5)
    sphere_ibc = {"segments": [segment("top", top, ["2", "0", "4"]),
                               segment("bottom", bottom, ["2", "-8", "5"])],
                  "ibcs": [["4", "cosine", "0", "0", "80", "10"],
                           ["5", "exp", "30", "0", "300", "-40"]]}
    # an impedance flag without a model: a PEC body
    sphere_unknown = {"segments": [segment("sphere", arc(6.0, 0.0, 0.0, 180.0, 12),
                                           ["2", "0", "7", "0", "0"])],
                      "ibcs": [["6", "constant", "10", "0", "0", "0"]]}
    # homogeneous dielectric bodies (TYPE 3): an inline lossless medium, and a
    # frequency table of eps and mu (tests/golden/materials/mat.53)
    diel = {"segments": [segment("d1", arc(6.0, 0.0, 0.0, 90.0, 6), ["3", "0", "0", "3", "0"]),
                         segment("d2", arc(6.0, 0.0, 90.0, 180.0, 6), ["3", "-10", "0", "3", "0"])],
            "dielectrics": [["3", "4.0", "0", "1.0", "0"]]}
    diel_table = {"segments": [segment("d", arc(0.15, 0.0, 0.0, 180.0, 9), ["3", "0", "0", "mat.53"])],
                  "dielectrics": [["53"]]}
    return {"sphere_in": sphere, "cone_sphere_m": cone_sphere, "ogive_in": ogive,
            "cone_sphere_ibc_m": cone_ibc, "sphere_ibc_in": sphere_ibc,
            "sphere_unknown_flag_in": sphere_unknown, "dielectric_sphere_in": diel,
            "dielectric_table_m": diel_table}


def cases():
    """(name, snapshot name, keyword arguments of solve_monostatic_rcs_bor)."""
    th = list(np.arange(0.0, 180.0001, 15.0))
    return [
        ("sphere_two_freqs", "sphere_in",
         dict(frequencies_ghz=[1.0, 2.5], elevations_deg=th, polarization="VV")),
        ("sphere_hh_one_freq", "sphere_in",
         dict(frequencies_ghz=[1.7], elevations_deg=th, polarization="horizontal",
              n_modes=9, mode_tol=0.0, table_precision="double")),
        ("cone_sphere_efie_360", "cone_sphere_m",
         dict(frequencies_ghz=[2.0, 3.0], elevations_deg=[0.0, 10.0, 45.0, 90.0, 180.0],
              polarization="HH", geometry_units="meters", mesh_reference_ghz=3.0,
              cfie_alpha=0.0, expand_to_360=True)),
        ("cone_sphere_per_freq_mesh", "cone_sphere_m",
         dict(frequencies_ghz=[0.5, 1.25, 4.0], elevations_deg=[30.0, 60.0],
              polarization="TE", geometry_units="m", cfie_alpha=0.3)),
        ("ogive", "ogive_in",
         dict(frequencies_ghz=[2.2], elevations_deg=th, polarization="", workers=3)),
        ("cone_sphere_ibc", "cone_sphere_ibc_m",
         dict(frequencies_ghz=[0.5, 2.0, 2.5, 4.0], elevations_deg=[0.0, 30.0, 90.0, 150.0],
              polarization="VV", geometry_units="meters", material_base_dir=MATERIALS)),
        ("sphere_ibc_tapers", "sphere_ibc_in",
         dict(frequencies_ghz=[1.0, 2.0], elevations_deg=th, polarization="HH",
              mesh_reference_ghz=2.0, expand_to_360=True, mode_tol=0.0)),
        ("sphere_ibc_single_freq", "sphere_ibc_in",
         dict(frequencies_ghz=[1.3], elevations_deg=[0.0, 90.0], polarization="VV", cfie_alpha=0.0)),
        ("sphere_unknown_impedance_flag", "sphere_unknown_flag_in",
         dict(frequencies_ghz=[1.5, 2.0], elevations_deg=[0.0, 90.0], polarization="VV",
              cfie_alpha=0.4)),
        ("dielectric_sphere", "dielectric_sphere_in",
         dict(frequencies_ghz=[1.0, 1.8], elevations_deg=[0.0, 45.0, 90.0], polarization="HH",
              n_modes=7, mode_tol=0.0)),
        ("dielectric_table", "dielectric_table_m",
         dict(frequencies_ghz=[0.5, 1.5, 2.5, 3.5], elevations_deg=[10.0, 170.0], polarization="VV",
              geometry_units="meters", material_base_dir=MATERIALS, expand_to_360=True)),
        ("dielectric_mesh_reference", "dielectric_sphere_in",
         dict(frequencies_ghz=[1.0, 2.0], elevations_deg=[30.0], polarization="VV",
              mesh_reference_ghz=1.5)),
    ]


def bad_inputs():
    """(name, snapshot, kwargs) the reference rejects."""
    snaps = snapshots()
    ok = snaps["sphere_in"]
    base = dict(frequencies_ghz=[1.0], elevations_deg=[0.0, 90.0], polarization="VV")
    arc_ = arc(6.0, 0.0, 0.0, 180.0, 6)
    seg = segment

    def with_segments(*segs):
        return {"segments": list(segs)}

    broken = copy.deepcopy(ok)
    broken["segments"][0]["point_pairs"][3]["x1"] += 0.5
    same_start = with_segments(seg("a", arc_[:4], ["2"]), seg("b", arc_[:2], ["2"]))
    reversed_piece = with_segments(seg("a", arc_[:4], ["2"]), seg("b", arc_[3:][::-1], ["2"]))
    loop = with_segments(seg("a", arc_, ["2"]),
                         seg("b", np.array([[1.0, 1.0], [2.0, 1.0], [2.0, 2.0], [1.0, 1.0]]),
                             ["2"]))
    closed_pair = with_segments(seg("a", arc_, ["2"]),
                                seg("b", np.array([arc_[-1], [-3.0, 0.0], arc_[0]]), ["2"]))
    crossing = with_segments(seg("a", np.vstack([arc_[:3], [[-2.0, 0.0]], arc_[4:]]), ["2"]))
    off_axis = with_segments(seg("a", arc_[:5], ["2"]))
    upward = with_segments(seg("a", arc_[::-1], ["2"]))
    sheet = with_segments(seg("a", arc_, ["1"]))
    mixed = with_segments(seg("a", arc_[:4], ["2"]), seg("b", arc_[3:], ["3", "0", "0", "1"]))
    two_media = with_segments(seg("a", arc_[:4], ["3", "0", "0", "1"]),
                              seg("b", arc_[3:], ["3", "0", "0", "2"]))
    aborted = threading.Event()
    aborted.set()

    def with_ibcs(ibcs, dielectrics=None):
        snap = copy.deepcopy(ok)
        snap["segments"][0]["properties"] = ["2", "0", "1", "0", "0"]
        snap["ibcs"] = ibcs
        if dielectrics is not None:
            snap["dielectrics"] = dielectrics
        return snap

    in_mat = dict(base, material_base_dir=MATERIALS)
    return [
        ("ibc_too_few_tokens", with_ibcs([["1", "linear", "1", "2"]]), base),
        ("ibc_unknown_taper", with_ibcs([["1", "spline", "1", "2", "3", "4"]]), base),
        ("ibc_nonfinite_taper", with_ibcs([["1", "linear", "1", "inf", "0", "0"]]), base),
        ("ibc_table_missing", with_ibcs([["77"]]), in_mat),
        ("ibc_table_nonfinite", with_ibcs([["52"]]), in_mat),
        ("dielectric_nonfinite", with_ibcs([], [["3", "nan", "0"]]), base),
        ("dielectric_table_missing", with_ibcs([], [["mat.78"]]), in_mat),
        ("no_frequencies", ok, dict(base, frequencies_ghz=[])),
        ("no_aspects", ok, dict(base, elevations_deg=[])),
        ("negative_frequency", ok, dict(base, frequencies_ghz=[1.0, -2.0])),
        ("aspect_above_180", ok, dict(base, elevations_deg=[0.0, 190.0])),
        ("bad_polarization", ok, dict(base, polarization="XX")),
        ("bad_units", ok, dict(base, geometry_units="cm")),
        ("no_segments", {"segments": []}, base),
        ("primitives_not_chained", broken, base),
        ("two_segments_same_start", same_start, base),
        ("reversed_segment", reversed_piece, base),
        ("separate_loop", loop, base),
        ("closed_polygon", closed_pair, base),
        ("crosses_axis", crossing, base),
        ("end_off_axis", off_axis, base),
        ("drawn_upward", upward, base),
        ("too_many_elements", ok, dict(base, frequencies_ghz=[40.0], max_elements=200)),
        ("sheet_type_1", sheet, base),
        ("pec_with_dielectric", mixed, base),
        ("dielectric_two_media", two_media, base),
        ("aborted", ok, dict(base, abort_event=aborted)),
    ]
