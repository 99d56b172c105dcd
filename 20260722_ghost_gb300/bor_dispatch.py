"""Drop-in replacement for the reference module ``bor_dispatch`` (PEC bodies).

Entry points with the reference's names, arguments and result layout:

  solve_monostatic_rcs_bor            bor_dispatch.py:335-702
  bor_az_el_grid                      bor_dispatch.py:705-828
  solve_adaptive_frequency_sweep_bor  bor_dispatch.py:831-925

A .geo geometry snapshot draws the generatrix in the (x, y) = (rho, z)
half-plane: a chain of segments, each a head-to-tail polyline, whose two ends
lie on the axis and which runs from the +z end to the -z end (the exterior is
left of travel).  The snapshot is checked and meshed on the host; every
frequency is then solved on the GPU by ``bor_solver.solve_bor``.  Several
frequencies go through ``bor_solver.solve_bor_batch``, which builds the next
frequency's problem on a host thread while the GPU sweeps the current one.

Scope: bodies whose segments are all TYPE 2 conductors -- PEC (CFIE, or EFIE
when cfie_alpha <= 0) and conductors with surface-impedance (IBC) flags,
whose Z_s per element comes from the snapshot's material tables
(materials.MaterialLibrary) and which are solved with the IBC-EFIE -- and
homogeneous TYPE 3 dielectric bodies (PMCHWT).
The multi-region kinds (TYPE 3+4 coated, TYPE 2+3+4 partial coating, TYPE
3+4+5 layered) are recognised and rejected with NotImplementedError;
malformed snapshots and material tables raise as in the reference.
"""

from __future__ import annotations

import cmath
import math
import os
import threading
from dataclasses import dataclass, field
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

from .bor_solver import solve_bor, solve_bor_batch, solve_bor_dielectric
from .geometry import C0
from .materials import MaterialLibrary

DEFAULT_ELEMENTS_PER_WAVELENGTH = 20
MAX_ELEMENTS_DEFAULT = 50_000

_NOT_ON_GPU = {
    "coated": "coated PEC bodies (multi-region PMCHWT)",
    "partial": "partially coated PEC bodies (PMCHWT with junctions)",
    "layered": "layered coated PEC bodies (PMCHWT)",
    "layered_n": "N-layer coated PEC bodies (PMCHWT)",
}


# ----------------------------------------------------------------------------
# snapshot parsing (bor_dispatch.py:38-131)
# ----------------------------------------------------------------------------

def _meters_per_unit(units: str) -> float:
    """Scale of the drawing units (bor_dispatch.py:38-44)."""
    u = str(units or "").strip().lower()
    if u in ("inch", "inches", "in"):
        return 0.0254
    if u in ("meter", "meters", "m"):
        return 1.0
    raise ValueError(f"Geometry units '{units}' are not supported; use inches or meters.")


def canonical_polarization(label: Optional[str]) -> str:
    """VV (theta-pol) or HH (phi-pol); the 2-D aliases TE -> VV and TM -> HH
    and an empty label (-> VV) as in bor_dispatch.py:47-58."""
    t = str(label or "").strip().upper()
    if not t or t in ("VV", "V", "TE", "VERTICAL"):
        return "VV"
    if t in ("HH", "H", "TM", "HORIZONTAL"):
        return "HH"
    raise ValueError(f"Polarization '{label}' is not supported; use VV or HH.")


def _number(tok: Any, default: int, strip_mat: bool) -> int:
    """A snapshot property as an integer: '', junk or None give ``default``;
    ``strip_mat`` accepts the 'mat.N' spelling of material flags
    (bor_dispatch.py:61-82)."""
    try:
        s = str(tok).strip()
        if strip_mat and s.lower().startswith("mat."):
            s = s[4:]
        return int(float(s)) if s else default
    except (TypeError, ValueError):
        return default


@dataclass
class Chain:
    """One snapshot segment as a polyline in metres (rows are (rho, z))."""
    name: str
    seg_type: int
    n_prop: int
    ibc_flag: int
    pos_mat: int
    neg_mat: int
    pts: np.ndarray
    prim_lengths: np.ndarray = field(init=False)
    length: float = field(init=False)

    def __post_init__(self):
        d = np.diff(self.pts, axis=0)
        self.prim_lengths = np.hypot(d[:, 0], d[:, 1])
        self.length = float(np.sum(self.prim_lengths))


def chains_from_snapshot(snapshot: Dict[str, Any], scale: float) -> List[Chain]:
    """Segments of a snapshot (``properties`` = [TYPE, N, ibc, pos_mat,
    neg_mat], ``point_pairs`` = primitives x1,y1 -> x2,y2) as chains; the
    primitives of one segment must join head to tail (bor_dispatch.py:85-131).
    Segments with fewer than two points are skipped."""
    out: List[Chain] = []
    for idx, seg in enumerate(snapshot.get("segments", []) or []):
        raw = list(seg.get("properties", []) or [])
        t0 = raw[0] if raw and str(raw[0]).strip() else seg.get("seg_type", 2)
        props = raw + [None] * 5            # absent properties parse to their defaults
        name = str(seg.get("name", f"segment_{idx + 1}"))
        pts: List[Tuple[float, float]] = []
        for j, pp in enumerate(seg.get("point_pairs", []) or []):
            a = (float(pp.get("x1", 0.0)) * scale, float(pp.get("y1", 0.0)) * scale)
            b = (float(pp.get("x2", 0.0)) * scale, float(pp.get("y2", 0.0)) * scale)
            if j and math.hypot(a[0] - pts[-1][0], a[1] - pts[-1][1]) > 0:
                raise ValueError(
                    f"Segment '{seg.get('name', idx)}': primitive {j} starts at "
                    f"({a[0] / scale:.6g}, {a[1] / scale:.6g}), not where the previous one ended.")
            if not j:
                pts.append(a)
            pts.append(b)
        if len(pts) >= 2:
            out.append(Chain(name, _number(t0, 2, True), _number(props[1], 0, False),
                             _number(props[2], 0, True), _number(props[3], 0, True),
                             _number(props[4], 0, True), np.asarray(pts, dtype=float)))
    if not out:
        raise ValueError("The geometry has no usable segments.")
    return out


def classify(chains: Sequence[Chain]) -> str:
    """Material kind of a snapshot from its segment TYPEs and material flags
    (bor_dispatch.py:232-280): 'conductor', 'dielectric', 'coated',
    'partial', 'layered' or 'layered_n'; any other mix raises ValueError."""
    types = {c.seg_type for c in chains}
    flags = lambda t, attr: {getattr(c, attr) for c in chains if c.seg_type == t}  # noqa: E731
    if types == {2}:
        return "conductor"
    if types == {3}:
        if len(flags(3, "pos_mat")) != 1:
            raise ValueError("A homogeneous body needs one pos_mat on all its TYPE 3 segments.")
        return "dielectric"
    if types in ({3, 4}, {2, 3, 4}):
        p3, p4 = flags(3, "pos_mat"), flags(4, "pos_mat")
        if len(p3) != 1 or p3 != p4:
            raise ValueError("A coated body needs the same single pos_mat on its TYPE 3 "
                             "interface and its TYPE 4 core.")
        return "partial" if 2 in types else "coated"
    if types == {3, 4, 5}:
        pairs = {(c.pos_mat, c.neg_mat) for c in chains if c.seg_type == 5}
        if len(pairs) > 1:
            return "layered_n"
        outer, inner = next(iter(pairs))
        if outer <= 0 or inner <= 0 or outer == inner:
            raise ValueError("A TYPE 5 interface needs two different positive flags "
                             "(pos_mat outer layer, neg_mat inner layer).")
        if flags(4, "pos_mat") != {inner}:
            raise ValueError("The TYPE 4 core's pos_mat must equal the TYPE 5 neg_mat.")
        if not flags(3, "pos_mat") <= {outer, inner}:
            raise ValueError("Each TYPE 3 pos_mat must be the outer or the inner layer flag.")
        return "layered"
    other = sorted(types - {2, 3, 4, 5})
    if other:
        raise ValueError(f"Segment TYPE(s) {other} cannot be solved as a body of revolution "
                         "(TYPE 2, 3, 3+4, 2+3+4 and 3+4+5 can).")
    raise ValueError("TYPE 2 conductors combine with dielectric segments only in the "
                     "TYPE 2+3+4 partial-coating layout.")


# ----------------------------------------------------------------------------
# generatrix: ordering, checks, mesh (bor_dispatch.py:134-229)
# ----------------------------------------------------------------------------

def _key(p: np.ndarray, tol: float) -> Tuple[int, int]:
    return (int(round(p[0] / tol)), int(round(p[1] / tol)))


def chain_runs(chains: Sequence[Chain], what: str, tol: float) -> List[List[Chain]]:
    """Maximal head-to-tail runs of ``chains``: a run starts at a chain whose
    start is no chain's end and follows end -> start matches (points equal to
    ``tol``), never reversing a chain, since that would flip its normal.
    Two chains that start (or end) at one point raise ValueError; chains on
    a closed loop belong to no run."""
    starts: Dict[Tuple[int, int], Chain] = {}
    ends: Dict[Tuple[int, int], Chain] = {}
    for c in chains:
        ks, ke = _key(c.pts[0], tol), _key(c.pts[-1], tol)
        if ks in starts or ke in ends:
            raise ValueError(f"Two {what} segments start or end at the same point; "
                             "the segments must form one head-to-tail chain.")
        starts[ks], ends[ke] = c, c
    runs = []
    for c in chains:
        if _key(c.pts[0], tol) in ends:
            continue
        run = [c]
        # unique starts and ends: a walk from a head can neither branch nor cycle
        while (nxt := starts.get(_key(run[-1].pts[-1], tol))) is not None:
            run.append(nxt)
        runs.append(run)
    return runs


def generatrix_run(chains: Sequence[Chain], what: str, tol: float) -> List[Chain]:
    """The chains as ONE head-to-tail run, in traversal order
    (bor_dispatch.py:134-183); anything else raises ValueError."""
    if len(chains) == 1:
        return list(chains)
    runs = chain_runs(chains, what, tol)
    if not runs:
        raise ValueError(f"The {what} segments close on themselves in the (rho, z) plane; a "
                         "generatrix is an open polyline with both ends on the axis.")
    if len(runs) > 1:
        raise ValueError(f"The {what} segments make {len(runs)} separate runs, not one "
                         "generatrix: consecutive segments must share end points and be drawn "
                         "in the same direction (reverse the end points of a segment that "
                         "meets its neighbour start-to-start or end-to-end).")
    if len(runs[0]) != len(chains):
        raise ValueError(f"Some {what} segments form a closed loop apart from the generatrix.")
    return runs[0]


def preflight(run: Sequence[Chain], what: str, axis_tol: float) -> None:
    """A closed body of revolution: rho >= 0 everywhere, both ends on the
    axis, traversed from the +z end to the -z end (bor_dispatch.py:186-206)."""
    pts = np.vstack([run[0].pts] + [c.pts[1:] for c in run[1:]])
    rho, z = pts[:, 0], pts[:, 1]
    if np.any(rho < -axis_tol):
        x = pts[np.argmin(rho), 0]
        raise ValueError(f"The {what} generatrix crosses the axis (rho = x = {x:.6g} < 0); "
                         "draw the half-profile at x >= 0.")
    if rho[0] > axis_tol or rho[-1] > axis_tol:
        raise ValueError(f"The {what} generatrix must start and end ON the axis (x = 0) to "
                         f"close the body; its ends are at rho = {rho[0]:.6g} and "
                         f"{rho[-1]:.6g}. Open shells are not supported.")
    if z[0] <= z[-1]:
        raise ValueError(f"The {what} generatrix runs from z = {z[0]:.6g} to {z[-1]:.6g}; draw "
                         "it from the +z axis end to the -z end (exterior on the left).")


def element_count(n_prop: int, prim_len: float, lam: float) -> int:
    """Elements of one primitive (bor_dispatch.py:209-216): N > 0 gives N
    elements, N < 0 gives |N| per wavelength, N = 0 the default density;
    at most 2000 per primitive."""
    if prim_len <= 0.0:
        return 1
    if n_prop > 0:
        return n_prop
    per_wave = -n_prop if n_prop < 0 else DEFAULT_ELEMENTS_PER_WAVELENGTH
    size = max(lam / per_wave, prim_len / 2000.0)
    return max(1, int(math.ceil(prim_len / size)))


def mesh_generatrix(run: Sequence[Chain], lam: float, max_elements: int,
                    axis_tol: float) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Nodes [Nn, 2] (rho, z) of the run, each primitive cut into equal
    elements, plus per element its chain index and the normalised arc
    position of its midpoint along that chain (the taper coordinate of an
    impedance flag), as bor_dispatch.py:219-229.  Coordinates within
    ``axis_tol`` of the axis are put on it."""
    nodes = [run[0].pts[:1].astype(float)]
    seg_of: List[np.ndarray] = []
    arc_of: List[np.ndarray] = []
    for ci, c in enumerate(run):
        arc0 = 0.0
        for p0, p1, plen in zip(c.pts[:-1], c.pts[1:], c.prim_lengths):
            cnt = element_count(c.n_prop, plen, lam)
            frac = np.arange(1, cnt + 1) / cnt
            nodes.append(p0 + (p1 - p0) * frac[:, None])
            seg_of.append(np.full(cnt, ci, dtype=int))
            arc_of.append((arc0 + plen * (np.arange(cnt) + 0.5) / cnt) / max(c.length, 1e-300))
            arc0 += plen
    pts = np.vstack(nodes)
    pts[np.abs(pts[:, 0]) <= axis_tol, 0] = 0.0
    pts[:, 0] = np.maximum(pts[:, 0], 0.0)
    if len(pts) - 1 > max_elements:
        raise ValueError(f"The mesh needs {len(pts) - 1} elements, more than max_elements = "
                         f"{max_elements}; lower the frequency or the density.")
    return pts, np.concatenate(seg_of), np.concatenate(arc_of)


def causal_index(eps_r: complex, mu_r: complex) -> complex:
    """Refractive index sqrt(eps_r mu_r) on the causal branch (Im <= 0, then
    Re >= 0), as the reference picks it (bor_solver.py:161-172)."""
    m = complex(np.sqrt(complex(eps_r) * complex(mu_r)))
    if m.imag > 0.0:
        m = -m
    if m.real < 0.0:
        m = -m
    return m


def prepare_snapshot(snapshot: Dict[str, Any], geometry_units: str = "inches"):
    """Parse, classify and check a snapshot.  Returns (kind, run, axis_tol)
    for a conductor or a homogeneous dielectric body; other kinds raise
    NotImplementedError."""
    chains = chains_from_snapshot(snapshot, _meters_per_unit(geometry_units))
    kind = classify(chains)
    if kind not in ("conductor", "dielectric"):
        raise NotImplementedError(f"{_NOT_ON_GPU[kind]} are not on the GPU path; "
                                  "conductors (TYPE 2) and homogeneous dielectric bodies (TYPE 3) are.")
    extent = np.ptp(np.vstack([c.pts for c in chains]), axis=0).max()
    diag = max(float(extent), 1e-9)
    run = generatrix_run(chains, "TYPE 2" if kind == "conductor" else "TYPE 3", max(1e-12, 1e-9 * diag))
    axis_tol = 1e-6 * diag
    preflight(run, "body", axis_tol)
    return kind, run, axis_tol


# ----------------------------------------------------------------------------
# monostatic sweep over frequencies (bor_dispatch.py:335-702)
# ----------------------------------------------------------------------------

def _samples_of(out: Dict[str, Any], freq_ghz: float, aspects: Sequence[float],
                pol: str) -> List[Dict[str, Any]]:
    """One sample row per aspect angle (bor_dispatch.py:640-656)."""
    sig = out["sigma_vv"] if pol == "VV" else out["sigma_hh"]
    amp = out["amp_vv"] if pol == "VV" else out["amp_hh"]
    residual = float(out.get("linear_residual", 0.0))
    rows = []
    for a, s, f in zip(aspects, sig, amp):
        lin = max(float(s), 1e-30)
        f = complex(f)
        rows.append({
            "frequency_ghz": float(freq_ghz), "theta_inc_deg": float(a),
            "theta_scat_deg": float(a), "rcs_linear": lin,
            "rcs_db": 10.0 * math.log10(lin),
            "rcs_amp_real": f.real, "rcs_amp_imag": f.imag,
            "rcs_amp_phase_deg": math.degrees(cmath.phase(f)),
            "linear_residual": residual,
        })
    return rows


def _mirror_to_360(samples: List[Dict[str, Any]]) -> List[Dict[str, Any]]:
    """sigma(360 - theta) = sigma(theta) for a body of revolution (a half
    turn about the axis maps body, look and polarisation basis onto
    themselves, complex amplitudes included); the seams 0 and 180 are not
    repeated (bor_dispatch.py:671-680)."""
    extra = []
    for s in samples:
        th = float(s["theta_inc_deg"])
        if 0.0 < th < 180.0:
            m = dict(s)
            m["theta_inc_deg"] = m["theta_scat_deg"] = 360.0 - th
            extra.append(m)
    return sorted(samples + extra, key=lambda s: (s["frequency_ghz"], s["theta_inc_deg"]))


def solve_monostatic_rcs_bor(
    geometry_snapshot: Dict[str, Any],
    frequencies_ghz: List[float],
    elevations_deg: List[float],
    polarization: str,
    geometry_units: str = "inches",
    material_base_dir: Optional[str] = None,
    progress_callback: Optional[Callable[[int, int, str], None]] = None,
    mesh_reference_ghz: Optional[float] = None,
    cfie_alpha: float = 0.5,
    n_modes: Optional[int] = None,
    mode_tol: float = 1e-6,
    max_elements: int = MAX_ELEMENTS_DEFAULT,
    workers: Optional[int] = None,
    abort_event: Optional[threading.Event] = None,
    table_precision: str = "auto",
    assembly: str = "auto",
    expand_to_360: bool = False,
) -> Dict[str, Any]:
    """Monostatic 3-D RCS (m^2, dBsm) of the body of revolution a .geo
    snapshot draws, at every frequency (GHz) and aspect angle (degrees from
    the +z axis: 0 nose-on, 90 broadside, 180 tail-on).

    Both polarisations are solved (each mode's factorisation serves both);
    ``polarization`` picks the one the samples report.  The body is meshed per
    frequency (or once at ``mesh_reference_ghz``) at the segments' densities,
    solved with the CFIE (EFIE when ``cfie_alpha`` <= 0) on the GPU, and the
    result has the reference's layout: ``samples`` rows plus ``metadata``
    (bor_dispatch.py:682-702).  ``expand_to_360`` adds the mirrored aspects
    360 - theta.  ``material_base_dir`` and ``workers`` are accepted for
    compatibility; ``abort_event`` is polled between frequencies.
    """
    if not frequencies_ghz:
        raise ValueError("At least one frequency is required.")
    if not elevations_deg:
        raise ValueError("At least one aspect angle is required.")
    freqs = [float(f) for f in frequencies_ghz]
    if any(f <= 0.0 for f in freqs):
        raise ValueError("Frequencies must be positive GHz values.")
    aspects = [float(a) for a in elevations_deg]
    if any(a < 0.0 or a > 180.0 for a in aspects):
        raise ValueError("Aspect angles must lie in [0, 180] degrees from +z.")
    pol = canonical_polarization(polarization)
    _meters_per_unit(geometry_units)
    if workers is None:
        workers = max(1, (os.cpu_count() or 2) - 1)
    # material tables first, as the reference reads them (bor_dispatch.py:389-393)
    materials = MaterialLibrary.from_entries(geometry_snapshot.get("ibcs", []) or [],
                                             geometry_snapshot.get("dielectrics", []) or [],
                                             base_dir=material_base_dir or os.getcwd())
    kind, run, axis_tol = prepare_snapshot(geometry_snapshot, geometry_units)
    form = "efie" if cfie_alpha <= 0.0 else "cfie"
    label = f"BoR-MoM PEC {form.upper()}"

    def check_abort():
        if abort_event is not None and abort_event.is_set():
            raise InterruptedError("Solve cancelled by user.")

    def notify(i, msg):
        if progress_callback is not None:
            try:
                progress_callback(i, len(freqs), msg)
            except Exception:                      # a failing callback never stops a solve
                pass

    def mesh(freq_ghz, full=False):
        ghz = float(mesh_reference_ghz) if mesh_reference_ghz else freq_ghz
        m = mesh_generatrix(run, C0 / (ghz * 1e9), max_elements, axis_tol)
        return m if full else m[0]

    common = dict(formulation=form, cfie_alpha=cfie_alpha, mode_tol=mode_tol,
                  table_precision=table_precision)
    if kind == "dielectric":
        # one PMCHWT solve per frequency, meshed for the wavelength inside the
        # medium (bor_dispatch.py:540-549)
        outs = []
        for fi, f in enumerate(freqs):
            check_abort()
            eps, mu = materials.get_medium(run[0].pos_mat, f)
            ghz = float(mesh_reference_ghz) if mesh_reference_ghz else f
            lam = C0 / (ghz * 1e9) / max(1.0, abs(causal_index(eps, mu)))
            pts = mesh_generatrix(run, lam, max_elements, axis_tol)[0]

            def report(done, cap, fi=fi, f=f):
                notify(fi, f"{f:g} GHz: mode {done}/{cap}")

            out = solve_bor_dielectric(pts, f * 1e9, aspects, eps, mu, n_modes=n_modes, mode_tol=mode_tol,
                                       workers=workers, progress=report, check_abort=check_abort)
            for w in out.get("warnings", []) or []:
                materials.warn_once(str(w))
            outs.append(out)
            notify(fi + 1, f"Solved {f:g} GHz")
        return _sweep_result(freqs, outs, aspects, pol, kind, "BoR-MoM PMCHWT (homogeneous dielectric)",
                             cfie_alpha, workers, materials, expand_to_360, warnings_done=True)
    if any(c.ibc_flag > 0 for c in run):
        # impedance flags: Z_s per element at each frequency (material warnings
        # in the reference's order), one IBC-EFIE solve per frequency
        # (bor_dispatch.py:504-537)
        outs = []
        for fi, f in enumerate(freqs):
            check_abort()
            pts, seg_of, arc_of = mesh(f, full=True)
            zs = np.zeros(len(pts) - 1, dtype=complex)
            for ei in range(len(zs)):
                c = run[seg_of[ei]]
                if c.ibc_flag > 0:
                    zs[ei] = materials.get_impedance(c.ibc_flag, f, arc_s=float(arc_of[ei]))
            has_ibc = bool(np.any(np.abs(zs) > 0.0))
            form_f = "efie" if (has_ibc or cfie_alpha <= 0.0) else "cfie"

            def report(done, cap, fi=fi, f=f):
                notify(fi, f"{f:g} GHz: mode {done}/{cap}")

            out = solve_bor(pts, f * 1e9, aspects, formulation=form_f, cfie_alpha=cfie_alpha,
                            zs=zs if has_ibc else None, n_modes=n_modes, mode_tol=mode_tol,
                            workers=workers, progress=report, check_abort=check_abort,
                            table_precision=table_precision, assembly=assembly)
            label = "BoR-MoM IBC-EFIE (Leontovich)" if has_ibc else f"BoR-MoM PEC {form_f.upper()}"
            for w in out.get("warnings", []) or []:
                materials.warn_once(str(w))
            outs.append(out)
            notify(fi + 1, f"Solved {f:g} GHz")
        return _sweep_result(freqs, outs, aspects, pol, kind, label, cfie_alpha, workers,
                             materials, expand_to_360, warnings_done=True)

    check_abort()
    if len(freqs) == 1:
        f0 = freqs[0]

        def report(done, cap):
            notify(0, f"{f0:g} GHz: mode {done}/{cap}")

        outs = [solve_bor(mesh(f0), f0 * 1e9, aspects, n_modes=n_modes, workers=workers,
                          progress=report, check_abort=check_abort, assembly=assembly,
                          **common)]
        notify(1, f"Solved {f0:g} GHz")
    else:
        bodies = [{"points": mesh(f), "freq_hz": f * 1e9, "n_modes": n_modes} for f in freqs]

        def done(i, _n):
            notify(i, f"Solved {freqs[i - 1]:g} GHz")
            check_abort()

        outs = solve_bor_batch(bodies, aspects, progress=done, **common)
    return _sweep_result(freqs, outs, aspects, pol, kind, label, cfie_alpha, workers, materials,
                         expand_to_360, warnings_done=False)


def _sweep_result(freqs, outs, aspects, pol, kind, label, cfie_alpha, workers,
                  materials: MaterialLibrary, expand_to_360: bool, warnings_done: bool):
    """The result layout of solve_monostatic_rcs_bor (bor_dispatch.py:640-702);
    the solves' warnings join the material warnings once each, in order."""
    samples: List[Dict[str, Any]] = []
    per_freq: List[Dict[str, Any]] = []
    for f, out in zip(freqs, outs):
        if not warnings_done:
            for w in out.get("warnings", []) or []:
                materials.warn_once(str(w))
        samples += _samples_of(out, f, aspects, pol)
        residual = float(out.get("linear_residual", 0.0))
        per_freq.append({
            "frequency_ghz": f, "modes_used": int(out["modes_used"]),
            "n_unknowns": int(out["n_unknowns"]), "linear_residual": residual,
            "max_cond": float(out["max_cond"]) if "max_cond" in out else None,
            "precision": out.get("precision"), "refine_iters": out.get("refine_iters"),
        })
    if expand_to_360:
        samples = _mirror_to_360(samples)
    return {
        "solver": "bor_mom_rcs",
        "scattering_mode": "monostatic",
        "polarization": pol,
        "polarization_export": pol,
        "rcs_log_unit": "dBsm",
        "rcs_linear_quantity": "sigma_3d",
        "samples": samples,
        "metadata": {
            "formulation": label,
            "geometry_kind": kind,
            "expanded_to_360": bool(expand_to_360),
            "per_frequency": per_freq,
            "cfie_alpha": float(cfie_alpha),
            "workers": int(workers),
            "warnings": list(materials.warnings),
        },
    }


# ----------------------------------------------------------------------------
# radar-frame (azimuth, elevation) grid (bor_dispatch.py:705-828)
# ----------------------------------------------------------------------------

def _amplitudes_by_frequency(res: Dict[str, Any]) -> Dict[float, Tuple[np.ndarray, np.ndarray]]:
    """{frequency: (aspects ascending, complex amplitudes)} of a result."""
    groups: Dict[float, List[Tuple[float, complex]]] = {}
    for s in res["samples"]:
        groups.setdefault(float(s["frequency_ghz"]), []).append(
            (float(s["theta_inc_deg"]), complex(s["rcs_amp_real"], s["rcs_amp_imag"])))
    out = {}
    for f, rows in groups.items():
        th = np.array([t for t, _ in rows])
        a = np.array([v for _, v in rows], dtype=complex)
        order = np.argsort(th, kind="stable")
        out[f] = (th[order], a[order])
    return out


def _look_vectors(az_deg: np.ndarray, el_deg: np.ndarray) -> np.ndarray:
    """Unit look directions [..., 3] (x = az 0 on the horizon, z up)."""
    a, e = np.radians(az_deg), np.radians(el_deg)
    return np.stack([np.cos(e) * np.cos(a), np.cos(e) * np.sin(a), np.sin(e)], axis=-1)


def _unit(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def bor_az_el_grid(res_vv: Dict[str, Any], res_hh: Dict[str, Any],
                   azimuths_deg, elevations_deg,
                   axis_az_deg: float = 0.0,
                   axis_el_deg: float = 0.0) -> Dict[str, Any]:
    """Radar-frame monostatic polarimetric grid over (azimuth, elevation)
    from the VV and HH aspect sweeps of one body (same frequencies).

    A monostatic look at a body of revolution sees only the aspect angle
    theta to the axis, and in its own meridian plane the scattering matrix
    is diagonal, diag(F_VV(theta), F_HH(theta)).  Each look's amplitudes are
    interpolated linearly (real and imaginary parts) in theta and the
    matrix is turned into the earth-vertical radar basis,
    S = M^T diag(F_VV, F_HH) M with M[i, j] = target basis_i . radar basis_j,
    giving radar VV, HH and the cross-pol VH that appears off the waterline.
    Looks along the axis (F_VV = F_HH) or straight up/down (radar H
    undefined) keep M = I.  ``axis_az_deg``/``axis_el_deg`` orient the axis
    in the earth frame.  The radar labels equal the solver's only for a
    vertical axis; for a horizontal axis the el = 0 cut has radar VV = the
    solver's HH.  Returns axes, ``theta_map_deg`` [n_az, n_el] and per
    channel ``amp``/``sigma`` arrays [n_az, n_el, n_freq].
    """
    if canonical_polarization(res_vv.get("polarization")) != "VV" or \
            canonical_polarization(res_hh.get("polarization")) != "HH":
        raise ValueError("Pass the VV result first and the HH result second.")
    az = np.atleast_1d(np.asarray(azimuths_deg, dtype=float))
    el = np.atleast_1d(np.asarray(elevations_deg, dtype=float))
    fv, fh = _amplitudes_by_frequency(res_vv), _amplitudes_by_frequency(res_hh)
    freqs = sorted(fv)
    if sorted(fh) != freqs:
        raise ValueError("The VV and HH results cover different frequencies.")

    A, E = np.meshgrid(az, el, indexing="ij")
    d = _look_vectors(A, E)                                   # [n_az, n_el, 3]
    ax = _look_vectors(np.float64(axis_az_deg), np.float64(axis_el_deg))
    theta = np.degrees(np.arccos(np.clip(d @ ax, -1.0, 1.0)))
    c = np.cross(ax, d)                                       # normal of the meridian plane
    r = np.cross(np.array([0.0, 0.0, 1.0]), d)                # radar horizontal
    moot = (np.linalg.norm(c, axis=-1) < 1e-9) | (np.linalg.norm(r, axis=-1) < 1e-9)
    with np.errstate(invalid="ignore", divide="ignore"):     # moot looks are replaced below
        h_t = _unit(c)
        v_t = _unit(np.cross(h_t, d))
        h_r = _unit(r)
        v_r = _unit(np.cross(h_r, d))
        dot = lambda p, q: np.sum(p * q, axis=-1)             # noqa: E731
        m00, m01, m10, m11 = dot(v_t, v_r), dot(v_t, h_r), dot(h_t, v_r), dot(h_t, h_r)
    m00[moot], m01[moot], m10[moot], m11[moot] = 1.0, 0.0, 0.0, 1.0

    amp = {ch: np.zeros(A.shape + (len(freqs),), dtype=complex) for ch in ("VV", "HH", "VH")}
    for kf, f in enumerate(freqs):
        Fv = np.interp(theta, fv[f][0], fv[f][1].real) + 1j * np.interp(theta, fv[f][0], fv[f][1].imag)
        Fh = np.interp(theta, fh[f][0], fh[f][1].real) + 1j * np.interp(theta, fh[f][0], fh[f][1].imag)
        amp["VV"][..., kf] = m00 ** 2 * Fv + m10 ** 2 * Fh
        amp["HH"][..., kf] = m01 ** 2 * Fv + m11 ** 2 * Fh
        amp["VH"][..., kf] = m00 * m01 * Fv + m10 * m11 * Fh
    return {
        "azimuths_deg": az.tolist(),
        "elevations_deg": el.tolist(),
        "frequencies_ghz": freqs,
        "axis_az_deg": float(axis_az_deg),
        "axis_el_deg": float(axis_el_deg),
        "theta_map_deg": theta,
        "amp": amp,
        "sigma": {ch: 4.0 * math.pi * np.abs(a) ** 2 for ch, a in amp.items()},
        "rcs_log_unit": "dBsm",
        "rcs_linear_quantity": "sigma_3d",
    }


# ----------------------------------------------------------------------------
# adaptive frequency sweep (bor_dispatch.py:831-925)
# ----------------------------------------------------------------------------

def solve_adaptive_frequency_sweep_bor(
    geometry_snapshot: Dict[str, Any],
    freq_start_ghz: float,
    freq_stop_ghz: float,
    elevations_deg: List[float],
    polarization: str,
    initial_points: int = 11,
    max_refinements: int = 3,
    db_threshold: float = 1.0,
    max_total_points: int = 201,
    **kwargs,
) -> Dict[str, Any]:
    """Broadband sweep: ``initial_points`` (>= 3) equally spaced seed
    frequencies, then up to ``max_refinements`` passes that add the midpoint
    of every neighbouring pair whose RCS differs by more than
    ``db_threshold`` dB at any aspect, until ``max_total_points``.
    Frequencies are keyed rounded to 1e-12 GHz, so none is solved twice.
    Each pass's new frequencies go to the GPU as one batch.  ``kwargs`` pass
    to ``solve_monostatic_rcs_bor``; a set ``abort_event`` stops refining."""
    if freq_start_ghz <= 0 or freq_stop_ghz <= 0:
        raise ValueError("Frequencies must be positive.")
    if freq_start_ghz >= freq_stop_ghz:
        raise ValueError("freq_start_ghz must be less than freq_stop_ghz.")
    initial_points = max(3, int(initial_points))
    rkey = lambda f: round(float(f), 12)                      # noqa: E731
    solved: Dict[float, List[Dict[str, Any]]] = {}
    every: List[Dict[str, Any]] = []

    def solve(fs: List[float]) -> None:
        if fs:
            res = solve_monostatic_rcs_bor(geometry_snapshot=geometry_snapshot,
                                           frequencies_ghz=fs, elevations_deg=elevations_deg,
                                           polarization=polarization, **kwargs)
            for s in res.get("samples", []):
                solved.setdefault(rkey(s["frequency_ghz"]), []).append(s)
                every.append(s)

    freqs = sorted({rkey(f) for f in np.linspace(freq_start_ghz, freq_stop_ghz, initial_points)})
    solve(freqs)
    passes = 0
    abort = kwargs.get("abort_event")
    for _ in range(max_refinements):
        if (abort is not None and abort.is_set()) or len(freqs) >= max_total_points:
            break
        mids = set()
        for aspect in elevations_deg:
            db = {}
            for f in freqs:
                hit = next((s for s in solved.get(rkey(f), [])
                            if abs(s["theta_inc_deg"] - aspect) < 0.01), None)
                if hit is not None:
                    db[f] = hit["rcs_db"]
            for f0, f1 in zip(freqs[:-1], freqs[1:]):
                if f0 in db and f1 in db and abs(db[f1] - db[f0]) > db_threshold:
                    mid = rkey(0.5 * (f0 + f1))
                    if mid not in solved and mid not in (f0, f1):
                        mids.add(mid)
        if not mids:
            break
        new = sorted(mids)[:max_total_points - len(freqs)]
        solve(new)
        freqs = sorted(set(freqs) | set(new))
        passes += 1
    pol = canonical_polarization(polarization)
    return {
        "solver": "bor_mom_rcs",
        "scattering_mode": "monostatic_adaptive",
        "polarization": pol,
        "polarization_export": pol,
        "rcs_log_unit": "dBsm",
        "rcs_linear_quantity": "sigma_3d",
        "samples": sorted(every, key=lambda s: (s["frequency_ghz"], s["theta_inc_deg"])),
        "metadata": {
            "formulation": "BoR adaptive frequency sweep",
            "initial_points": initial_points,
            "final_point_count": len(freqs),
            "refinement_count": passes,
            "db_threshold": db_threshold,
            "freq_start_ghz": freq_start_ghz,
            "freq_stop_ghz": freq_stop_ghz,
        },
    }
