"""``.grim`` export of body-of-revolution results (reference module
``grim_io``: export_result_to_grim grim_io.py:210-262, save_bor_az_el_grim
grim_io.py:265-311) and its dBke CSV export (grim_io.py:50-78, 314-377).

A ``.grim`` file is a NumPy ``.npz`` archive: axes ``azimuths``,
``elevations``, ``frequencies`` (float64), ``polarizations`` (one label),
float32 grids [n_az, n_el, n_freq, n_pol] ``rcs_power`` (linear RCS),
``rcs_phase`` (radians) and optionally ``rcs_amp_real``/``rcs_amp_imag``,
plus string/bool metadata (units JSON, polarisation aliases, domain labels).
Empty cells are NaN.  The archive layout, key names and label strings are
the reference's, so files written here open in its viewers unchanged.
"""

from __future__ import annotations

import cmath
import json
import math
import os
from typing import Any, Dict, List, Optional

import numpy as np

_TINY = 1e-12
_TE_ALIASES = ["TE", "VV", "V", "VERTICAL"]
_TM_ALIASES = ["TM", "HH", "H", "HORIZONTAL"]


def _pol_2d(label: Optional[str]) -> str:
    """Elevation-cut label of a polarisation (TM = HH, TE = VV; empty -> TM)
    as grim_io.py:12-23."""
    t = str(label or "").strip().upper()
    if t in ("TM", "HH", "H", "HORIZONTAL") or not t:
        return "TM"
    if t in ("TE", "VV", "V", "VERTICAL"):
        return "TE"
    raise ValueError(f"Polarization '{label}' is not supported; use TM/HH/H/HORIZONTAL "
                     "or TE/VV/V/VERTICAL.")


def _grim_path(path: str) -> str:
    return path if path.lower().endswith(".grim") else path + ".grim"


def _incidence_tag(theta_inc_deg: float) -> str:
    """File-name tag of a bistatic incidence angle: inc_30p5, inc_m10."""
    v = f"{theta_inc_deg:.6f}".rstrip("0").rstrip(".")
    return "inc_" + (v.replace("-", "m").replace(".", "p") or "0")


def _write(payload: Dict[str, Any], path: str) -> str:
    """Write one archive; keys in the reference's order (grim_io.py:183-207)."""
    out = _grim_path(path)
    keys = ["azimuths", "elevations", "frequencies", "polarizations",
            "polarization_alias_primary", "polarization_aliases_json", "rcs_power",
            "rcs_phase", "rcs_domain", "power_domain", "source_path", "history", "units",
            "phase_reference", "raw_complex_amplitude_preserved"]
    defaults = {"polarization_alias_primary": "", "polarization_aliases_json": "",
                "raw_complex_amplitude_preserved": False}
    arrays = {k: payload[k] if k in payload or k not in defaults else defaults[k] for k in keys}
    if "rcs_amp_real" in payload and "rcs_amp_imag" in payload:
        arrays["rcs_amp_real"] = payload["rcs_amp_real"]
        arrays["rcs_amp_imag"] = payload["rcs_amp_imag"]
        arrays["complex_field_domain"] = payload.get("complex_field_domain",
                                                     "solver_raw_far_field_amplitude")
    with open(out, "wb") as fh:
        np.savez(fh, **arrays)
    return out


def _cut_payload(samples: List[Dict[str, Any]], polarization: str, source_path: str,
                 history: str, keep_amplitude: bool, log_unit: str,
                 linear_quantity: str) -> Dict[str, Any]:
    """Grid of one aspect cut: azimuth axis = theta_scat, one elevation (0),
    frequencies ascending, one polarisation (grim_io.py:80-180).  A repeated
    (angle, frequency) must repeat the same power and phase, else ValueError."""
    if not samples:
        raise ValueError("No samples available to export.")
    az = np.array(sorted({float(s["theta_scat_deg"]) for s in samples}), dtype=float)
    fr = np.array(sorted({float(s["frequency_ghz"]) for s in samples}), dtype=float)
    label = _pol_2d(polarization)
    ia = {v: i for i, v in enumerate(az)}
    jf = {v: i for i, v in enumerate(fr)}
    shape = (len(az), 1, len(fr), 1)
    power = np.full(shape, np.nan, dtype=np.float32)
    phase = np.full(shape, np.nan, dtype=np.float32)
    re = np.full(shape, np.nan, dtype=np.float32)
    im = np.full(shape, np.nan, dtype=np.float32)
    finite = lambda x: x if math.isfinite(x) else 0.0        # noqa: E731
    for s in samples:
        a, f = float(s["theta_scat_deg"]), float(s["frequency_ghz"])
        lin = float(s.get("rcs_linear", 0.0))
        lin = lin if math.isfinite(lin) and lin >= 0.0 else 0.0
        amp = complex(finite(float(s.get("rcs_amp_real", 0.0))),
                      finite(float(s.get("rcs_amp_imag", 0.0))))
        ph = float(cmath.phase(amp)) if abs(amp) > _TINY else 0.0
        cell = (ia[a], 0, jf[f], 0)
        if not np.isnan(power[cell]):
            if abs(power[cell] - lin) > _TINY:
                raise ValueError(f"Duplicate sample conflict at az={a}, el=0, f={f}, "
                                 f"pol={polarization}.")
            if np.isfinite(phase[cell]):
                # phases compared modulo 2 pi, to the float32 storage precision
                gap = (ph - float(phase[cell]) + math.pi) % (2.0 * math.pi) - math.pi
                if abs(gap) > 1e-5:
                    raise ValueError(f"Duplicate amplitude conflict at az={a}, el=0, f={f}, "
                                     f"pol={polarization}.")
            continue
        power[cell], phase[cell], re[cell], im[cell] = lin, ph, amp.real, amp.imag
    units = {"azimuth": "deg", "elevation": "deg", "frequency": "GHz",
             "rcs_log_unit": str(log_unit), "rcs_linear_quantity": str(linear_quantity)}
    payload = {
        "azimuths": az, "elevations": np.array([0.0]), "frequencies": fr,
        "polarizations": np.array(["HH" if label == "TM" else "VV"], dtype=str),
        "polarization_alias_primary": label,
        "polarization_aliases_json": json.dumps(_TM_ALIASES if label == "TM" else _TE_ALIASES),
        "rcs_power": power, "rcs_phase": phase,
        "rcs_domain": "power_phase", "power_domain": "linear_rcs",
        "source_path": source_path, "history": history, "units": json.dumps(units),
        "phase_reference": "origin=(0,0), convention=exp(+jwt), monostatic far-field amplitude",
        "raw_complex_amplitude_preserved": bool(keep_amplitude),
    }
    if keep_amplitude:
        payload.update(rcs_amp_real=re, rcs_amp_imag=im,
                       complex_field_domain="solver_raw_far_field_amplitude")
    return payload


def export_result_to_grim(result: Dict[str, Any], output_path: str,
                          polarization: Optional[str] = None, source_path: str = "",
                          history: str = "",
                          preserve_raw_complex_amplitude: bool = True) -> List[str]:
    """Write a solver result's samples as ``.grim``: one file for a
    monostatic result, one per incidence angle (``<root>_inc_<angle>.grim``)
    for a bistatic one.  Units come from the result (sigma_3d / dBsm for a
    body of revolution).  Returns the absolute paths written."""
    samples = result.get("samples", []) or []
    if not samples:
        raise ValueError("No solver samples were returned, nothing to export.")
    pol = _pol_2d(polarization or result.get("polarization_export")
                  or result.get("polarization") or "TM")
    units = (str(result.get("rcs_log_unit", "dBke")),
             str(result.get("rcs_linear_quantity", "sigma_2d")))
    if str(result.get("scattering_mode", "monostatic")).strip().lower() != "bistatic":
        p = _cut_payload(samples, pol, source_path, history,
                         preserve_raw_complex_amplitude, *units)
        return [os.path.abspath(_write(p, output_path))]
    by_inc: Dict[float, List[Dict[str, Any]]] = {}
    for s in samples:
        by_inc.setdefault(float(s.get("theta_inc_deg", 0.0)), []).append(s)
    root = _grim_path(output_path)[:-5]
    out = []
    for inc in sorted(by_inc):
        p = _cut_payload(by_inc[inc], pol, source_path,
                         (history + f" | theta_inc_deg={inc:g}").strip(" |"),
                         preserve_raw_complex_amplitude, *units)
        out.append(os.path.abspath(_write(p, f"{root}_{_incidence_tag(inc)}.grim")))
    return out


def save_bor_az_el_grim(grid: Dict[str, Any], output_path: str,
                        source_path: str = "", history: str = "") -> List[str]:
    """Write a ``bor_az_el_grid`` result as three ``.grim`` files
    (``<root>_VV``, ``_HH``, ``_VH``), each with real azimuth and elevation
    axes, sigma_3d power, phase and the complex amplitudes."""
    az = np.asarray(grid["azimuths_deg"], dtype=float)
    el = np.asarray(grid["elevations_deg"], dtype=float)
    fr = np.asarray(grid["frequencies_ghz"], dtype=float)
    root = _grim_path(output_path)[:-5]
    units = json.dumps({"azimuth": "deg", "elevation": "deg", "frequency": "GHz",
                        "rcs_log_unit": "dBsm", "rcs_linear_quantity": "sigma_3d"})
    aliases = {"VV": _TE_ALIASES, "HH": _TM_ALIASES, "VH": ["VH", "HV"]}
    tag = f"bor_az_el_grid axis_az={grid['axis_az_deg']:g} axis_el={grid['axis_el_deg']:g}"
    out = []
    for ch in ("VV", "HH", "VH"):
        a = np.asarray(grid["amp"][ch])[..., None]
        payload = {
            "azimuths": az, "elevations": el, "frequencies": fr,
            "polarizations": np.array([ch], dtype=str),
            "polarization_alias_primary": ch,
            "polarization_aliases_json": json.dumps(aliases[ch]),
            "rcs_power": (4.0 * math.pi * np.abs(a) ** 2).astype(np.float32),
            "rcs_phase": np.angle(a).astype(np.float32),
            "rcs_domain": "power_phase", "power_domain": "linear_rcs",
            "source_path": source_path,
            "history": (history + " | " + tag).strip(" |"),
            "units": units,
            "phase_reference": "origin=(0,0), convention=exp(+jwt), monostatic radar-frame "
                               "amplitude",
            "raw_complex_amplitude_preserved": True,
            "rcs_amp_real": a.real.astype(np.float32),
            "rcs_amp_imag": a.imag.astype(np.float32),
            "complex_field_domain": "solver_raw_far_field_amplitude",
        }
        out.append(os.path.abspath(_write(payload, f"{root}_{ch}")))
    return out


# ---------------------------------------------------------------------------
# dBke (knife-edge normalised scattering width) CSV export (grim_io.py:40-78, 314-377)
# ---------------------------------------------------------------------------

C0 = 299_792_458.0
_HZ_PER = {"hz": 1.0, "khz": 1.0e3, "mhz": 1.0e6, "ghz": 1.0e9}


def _to_hz(value: float, unit: str = "GHz") -> float:
    return float(value) * _HZ_PER.get(str(unit or "GHz").strip().lower(), 1.0e9)


def compute_dbke_from_linear(rcs_linear: float, frequency_value: float,
                             frequency_unit: str = "GHz") -> float:
    """Absolute dBke of a linear 2-D scattering width: 10 log10(k sigma_2d),
    k = 2 pi f / c0; non-finite or non-positive widths count as 1e-12."""
    lin = float(rcs_linear)
    if not math.isfinite(lin) or lin <= 0.0:
        lin = _TINY
    f = _to_hz(frequency_value, frequency_unit)
    if not math.isfinite(f) or f <= 0.0:
        raise ValueError("frequency_value must be a positive finite frequency.")
    return 10.0 * math.log10(((2.0 * math.pi * f) / C0) * lin)


def compute_linear_from_dbke(dbke_value: float, frequency_value: float,
                             frequency_unit: str = "GHz") -> float:
    """The linear 2-D scattering width of an absolute dBke value."""
    f = _to_hz(frequency_value, frequency_unit)
    if not math.isfinite(f) or f <= 0.0:
        raise ValueError("frequency_value must be a positive finite frequency.")
    return (C0 / (2.0 * math.pi * f)) * (10.0 ** (float(dbke_value) / 10.0))


def export_result_to_dbke_csv(result: Dict[str, Any], output_path: str, source_path: str = "",
                              history: str = "") -> str:
    """Write the samples, sorted by (frequency, incidence, scattering angle),
    as CSV with an absolute dBke column (a 2-D quantity; kept so the module
    is a complete stand-in for the reference's)."""
    samples = result.get("samples", []) or []
    if not samples:
        raise ValueError("No solver samples were returned, nothing to export.")
    out = output_path if output_path.lower().endswith(".csv") else output_path + ".csv"
    key = lambda r: (float(r.get("frequency_ghz", 0.0)), float(r.get("theta_inc_deg", 0.0)),  # noqa: E731
                     float(r.get("theta_scat_deg", 0.0)))
    cols = ["frequency_ghz", "theta_inc_deg", "theta_scat_deg", "rcs_linear", "rcs_db", "dbke",
            "rcs_amp_real", "rcs_amp_imag", "rcs_amp_phase_deg", "source_path", "history"]
    g = lambda v: f"{float(v):.12g}"                                                              # noqa: E731
    with open(out, "w", encoding="utf-8", newline="") as fh:
        fh.write(",".join(cols) + "\n")
        for r in sorted(samples, key=key):
            lin = float(r.get("rcs_linear", 0.0))
            if not math.isfinite(lin) or lin <= 0.0:
                lin = _TINY
            f = float(r.get("frequency_ghz", 0.0))
            db = float(r.get("rcs_db", 10.0 * math.log10(lin)))
            fh.write(",".join([g(f), g(r.get("theta_inc_deg", 0.0)), g(r.get("theta_scat_deg", 0.0)),
                               g(lin), g(db), g(compute_dbke_from_linear(lin, f, "GHz")),
                               g(r.get("rcs_amp_real", 0.0)), g(r.get("rcs_amp_imag", 0.0)),
                               g(r.get("rcs_amp_phase_deg", 0.0)), source_path.replace(",", ";"),
                               history.replace(",", ";")]) + "\n")
    return os.path.abspath(out)
