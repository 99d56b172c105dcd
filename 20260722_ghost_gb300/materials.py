"""Material tables of a .geo snapshot, as the BoR dispatch reads them.

The snapshot's ``ibcs`` rows give surface impedances Z_s per flag and its
``dielectrics`` rows (eps_r, mu_r) per flag; the reference keeps both in
``rcs_solver.MaterialLibrary`` (rcs_solver.py:303-460, with the parsers at
rcs_solver.py:769-856 and the models at rcs_solver.py:195-290).  Same rules
here, so that the impedance per element that reaches the GPU solve, the
warnings and the errors are the reference's:

* a flag (``"3"``, ``"mat.3"``, ``"3.0"``; anything else counts as 0) <= 0 is
  ignored; flags above 50 name a table file ``mat.<flag>`` in the material
  directory (else the working directory), rows ``f_GHz re im`` (impedance)
  or ``f_GHz eps' eps'' mu' mu''`` (medium), '#' comments, short or
  non-numeric rows skipped, non-finite values an error, sorted by frequency
  with the last row of a repeated frequency kept, sampled by linear
  interpolation of the real and imaginary parts (held constant outside the
  table, with a warning);
* inline impedance rows are ``flag kind R0 X0 R1 X1``: a Z_s that varies
  along the segment (arc position s in [0, 1] from its first point),
  ``constant``, ``linear``, ``cosine`` (raised-cosine weight) or ``exp``
  (geometric, zero ends floored at 1e-12);
* inline medium rows are ``flag eps' eps'' mu' mu''`` (missing entries:
  1, 0, 1, 0); a non-finite or (near-)zero value falls back to 1.
"""

from __future__ import annotations

import cmath
import math
import os
from dataclasses import dataclass
from typing import Any, Dict, List, Optional, Tuple, Union

import numpy as np

_FLOOR = 1e-12
_TAPER_KINDS = ("constant", "linear", "cosine", "exp")


def parse_flag(token: Any) -> int:
    text = str(token).strip().lower()
    if not text:
        return 0
    if text.startswith("mat."):
        text = text[4:]
    try:
        return int(float(text))
    except ValueError:
        return 0


def _float_or(token: Any, default: float) -> float:
    try:
        return float(token)
    except (TypeError, ValueError):
        return default


def _finite(z: complex, what: str) -> complex:
    z = complex(z)
    if not (math.isfinite(z.real) and math.isfinite(z.imag)):
        raise ValueError(f"{what} contains non-finite value {z!r}.")
    return z


def _or_unity(z: complex) -> complex:
    if not (math.isfinite(z.real) and math.isfinite(z.imag)) or abs(z) < _FLOOR:
        return 1.0 + 0.0j
    return z


def _table_file(base_dir: str, flag: int) -> str:
    name = f"mat.{flag}"
    for folder in (base_dir, os.getcwd()):
        path = os.path.join(folder, name)
        if os.path.isfile(path):
            return path
    raise FileNotFoundError(f"Could not locate material file {name} in {base_dir} or current directory.")


def _table_rows(path: str, ncol: int) -> List[List[float]]:
    rows: List[List[float]] = []
    with open(path, "r") as fh:
        for lineno, raw in enumerate(fh, start=1):
            tok = raw.split("#", 1)[0].split()
            if len(tok) < ncol:
                continue
            try:
                vals = [float(t) for t in tok[:ncol]]
            except ValueError:
                continue
            if not all(math.isfinite(v) for v in vals):
                raise ValueError(f"Material file '{path}' line {lineno} contains non-finite "
                                 f"numeric value(s): {tok[:ncol]}.")
            rows.append(vals)
    if not rows:
        raise ValueError(f"No valid numeric rows found in {path}")
    by_freq: Dict[float, List[float]] = {}
    for r in sorted(rows, key=lambda r: r[0]):
        by_freq[r[0]] = r
    return [by_freq[f] for f in sorted(by_freq)]


def _interp(f: float, fs: np.ndarray, vals: np.ndarray) -> complex:
    if len(fs) == 1:
        return complex(vals[0])
    return complex(np.interp(f, fs, vals.real), np.interp(f, fs, vals.imag))


@dataclass
class ImpedanceTable:
    """Z_s(f) from a mat.<flag> file."""
    freqs_ghz: np.ndarray
    values: np.ndarray

    @classmethod
    def load(cls, path: str) -> "ImpedanceTable":
        rows = _table_rows(path, 3)
        return cls(np.array([r[0] for r in rows]), np.array([complex(r[1], r[2]) for r in rows]))

    def sample(self, freq_ghz: float) -> complex:
        return _interp(freq_ghz, self.freqs_ghz, self.values)


@dataclass
class MediumTable:
    """(eps_r(f), mu_r(f)) from a mat.<flag> file."""
    freqs_ghz: np.ndarray
    eps: np.ndarray
    mu: np.ndarray

    @classmethod
    def load(cls, path: str) -> "MediumTable":
        rows = _table_rows(path, 5)
        return cls(np.array([r[0] for r in rows]), np.array([complex(r[1], r[2]) for r in rows]),
                   np.array([complex(r[3], r[4]) for r in rows]))

    def sample(self, freq_ghz: float) -> Tuple[complex, complex]:
        return _interp(freq_ghz, self.freqs_ghz, self.eps), _interp(freq_ghz, self.freqs_ghz, self.mu)


@dataclass
class ImpedanceTaper:
    """Z_s along one segment, s in [0, 1] from the segment's first point."""
    kind: str
    z_start: complex
    z_end: complex

    def __post_init__(self):
        if self.kind not in _TAPER_KINDS:
            raise ValueError(f"Unknown impedance taper kind '{self.kind}'. Expected one of {_TAPER_KINDS}.")
        self.z_start = _finite(self.z_start, "taper z_start")
        self.z_end = self.z_start if self.kind == "constant" else _finite(self.z_end, "taper z_end")

    def evaluate(self, s: float) -> complex:
        s = float(min(1.0, max(0.0, s)))
        if self.kind == "constant":
            return self.z_start
        if self.kind in ("linear", "cosine"):
            w = s if self.kind == "linear" else 0.5 * (1.0 - math.cos(math.pi * s))
            return (1.0 - w) * self.z_start + w * self.z_end
        za = self.z_start if abs(self.z_start) > _FLOOR else complex(_FLOOR, 0.0)
        zb = self.z_end if abs(self.z_end) > _FLOOR else complex(_FLOOR, 0.0)
        return cmath.exp((1.0 - s) * cmath.log(za) + s * cmath.log(zb))


class MaterialLibrary:
    """Impedance and medium models by flag, plus the warnings of their use."""

    def __init__(self, impedance: Dict[int, Union[ImpedanceTable, ImpedanceTaper]],
                 media: Dict[int, Union[Tuple[complex, complex], MediumTable]]):
        self.impedance_models = impedance
        self.dielectric_models = media
        self.warnings: List[str] = []

    @classmethod
    def from_entries(cls, ibcs_entries, dielectric_entries, base_dir: str) -> "MaterialLibrary":
        imp: Dict[int, Union[ImpedanceTable, ImpedanceTaper]] = {}
        med: Dict[int, Union[Tuple[complex, complex], MediumTable]] = {}
        for row in ibcs_entries:
            if not row:
                continue
            flag = parse_flag(row[0])
            if flag <= 0:
                continue
            if flag > 50:
                imp[flag] = ImpedanceTable.load(_table_file(base_dir, flag))
                continue
            tok = [str(t).strip() for t in row[1:] if str(t).strip() != ""]
            if len(tok) != 5:
                raise ValueError(f"IBC flag {flag}: inline impedance requires "
                                 f"'<kind> R_start X_start R_end X_end' (got {len(tok)} data tokens "
                                 "after the flag).")
            r0, x0, r1, x1 = (_float_or(t, 0.0) for t in tok[1:])
            imp[flag] = ImpedanceTaper(tok[0].lower(), complex(r0, x0), complex(r1, x1))
        for row in dielectric_entries:
            if not row:
                continue
            flag = parse_flag(row[0])
            if flag <= 0:
                continue
            if flag > 50:
                med[flag] = MediumTable.load(_table_file(base_dir, flag))
                continue
            v = [_float_or(row[i] if len(row) > i else d, d) for i, d in ((1, 1.0), (2, 0.0), (3, 1.0), (4, 0.0))]
            eps = _finite(complex(v[0], v[1]), f"Dielectric flag {flag} epsilon")
            mu = _finite(complex(v[2], v[3]), f"Dielectric flag {flag} mu")
            med[flag] = (_or_unity(eps), _or_unity(mu))
        return cls(imp, med)

    def warn_once(self, message: str) -> None:
        if message not in self.warnings:
            self.warnings.append(message)

    def _range_check(self, what: str, flag: int, freq_ghz: float, fs: np.ndarray) -> None:
        lo, hi = float(np.min(fs)), float(np.max(fs))
        if freq_ghz < lo or freq_ghz > hi:
            self.warn_once(f"{what} flag {flag} sampled at {freq_ghz:g} GHz outside table range "
                           f"[{lo:g}, {hi:g}] GHz.")

    def get_impedance(self, flag: int, freq_ghz: float, arc_s: Optional[float] = None) -> complex:
        """Z_s of an impedance flag at a frequency and arc position (0.5 when
        not given); 0 (PEC) for flags <= 0 and flags without a model."""
        model = self.impedance_models.get(flag) if flag > 0 else None
        if model is None:
            return 0.0 + 0.0j
        if isinstance(model, ImpedanceTable):
            self._range_check("Impedance", flag, freq_ghz, model.freqs_ghz)
            return _finite(model.sample(freq_ghz), f"IBC flag {flag} impedance sampled at {freq_ghz:g} GHz")
        s = 0.5 if arc_s is None else float(arc_s)
        return _finite(model.evaluate(s), f"IBC flag {flag} tapered impedance at s={s:g}")

    def is_tapered_impedance(self, flag: int) -> bool:
        return isinstance(self.impedance_models.get(flag), ImpedanceTaper)

    def get_medium(self, flag: int, freq_ghz: float) -> Tuple[complex, complex]:
        """(eps_r, mu_r) of a medium flag; free space for flags <= 0 and flags
        without a model."""
        model = self.dielectric_models.get(flag) if flag > 0 else None
        if model is None:
            return 1.0 + 0.0j, 1.0 + 0.0j
        if isinstance(model, MediumTable):
            self._range_check("Dielectric", flag, freq_ghz, model.freqs_ghz)
            eps, mu = model.sample(freq_ghz)
        else:
            eps, mu = model
        return _or_unity(eps), _or_unity(mu)
