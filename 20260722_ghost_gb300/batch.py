"""Batched sweeps of many bodies on one GPU: size classes, one factorisation
for all modes of all bodies of a class, CUDA-graph replay, and the autotuner.

The reference solves bodies one after another and, inside a body, waves of
|m| on CPU threads (run_local_bor.py:175-200, bor_solver.py:776-796).  Here:

* Size classes.  Bodies are sorted by their unknown count n and grouped so that
  every body of a class pads to the same n_pad (a multiple of the class width,
  chosen by the autotuner) and the class fits the memory budget.  Padded rows
  and columns of a mode system are identity rows and columns (as the masked
  axis unknowns are), so the padded unknowns come out exactly zero and every
  body's solution is that of its own system.
* One launch sequence per class.  The fills, the excitation, the exact first
  residual and the far field run per body (their kernels are persistent over
  element pairs and fill the GPU on their own) but write into the class's
  shared operator, right-hand-side and solution arrays; the LU, the
  substitutions and the residual updates then run once for all modes of all
  bodies of the class (batch = sum of M_i + 1), which keeps every SM busy where
  one small body would leave most of them idle.
* A fixed refinement schedule (one correction updated with exact products,
  the rest on the tensor-core GEMM) and no host synchronisation inside the
  sweep, so each class's whole sweep is captured once as a CUDA graph and
  replayed: a repeated sweep of the same bodies (new angles or a frequency
  step written into the same buffers) costs one graph launch per class.
* Autotuner (Autotuner below): per size class -- keyed by (device, n bucket,
  n_xi bucket, M bucket) -- it times the candidate class widths and near-fill
  grids on the class's first body and keeps the fastest in a JSON cache.

No counterpart in the reference.
"""

from __future__ import annotations

import json
import math
import os
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

from . import _native as nat
from .engine import BorGpuProblem, SweepResult

_HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_CACHE = os.path.join(_HERE, "_build", "autotune.json")


# ---------------------------------------------------------------------------
# autotuner
# ---------------------------------------------------------------------------
class Autotuner:
    """Picks, per size class, the padding width of the class and the near
    fill's persistent grid (CTAs per SM) by timing the candidates, and caches
    the choice as JSON (one entry per device name and size bucket)."""

    WIDTHS = (128, 256, 512)
    NEAR_GRIDS = (1, 2, 3)

    def __init__(self, path: Optional[str] = DEFAULT_CACHE):
        self.path = path
        self.table: Dict[str, Dict] = {}
        if path and os.path.exists(path):
            try:
                self.table = json.load(open(path))
            except (OSError, ValueError):
                self.table = {}

    @staticmethod
    def key(device_name: str, n: int, n_xi: int, m_max: int) -> str:
        nb = 1 << max(0, int(math.ceil(math.log2(max(n, 1)))))
        mb = 1 << max(0, int(math.ceil(math.log2(max(m_max + 1, 1)))))
        return f"{device_name}|n{nb}|nxi{n_xi}|m{mb}"

    def save(self):
        if not self.path:
            return
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.table, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)

    def near_grid(self, prob: BorGpuProblem) -> int:
        """CTAs per SM of the near fill for this body's size bucket (measured once)."""
        torch = prob.torch
        k = self.key(torch.cuda.get_device_name(prob.device), prob.n, prob.n_xi, prob.m_max)
        ent = self.table.setdefault(k, {})
        if "near_grid" not in ent:
            st = nat.stream_handle()
            band = torch.zeros((prob.m_max + 1, 4, prob.Nn, 5), dtype=torch.complex128, device=prob.device)
            times = {}
            lib = nat.load()
            try:
                for g in self.NEAR_GRIDS:
                    lib.ghost_bor_set_near_grid(g)
                    prob.fill_near(1.0 + 0.0j, st, band=band, precision=nat.F32)      # warm (workspace)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    prob.fill_near(1.0 + 0.0j, st, band=band, precision=nat.F32)
                    e1.record()
                    torch.cuda.synchronize()
                    times[g] = e0.elapsed_time(e1)
            finally:
                lib.ghost_bor_set_near_grid(0)
            ent["near_grid"] = min(times, key=times.get)
            ent["near_grid_ms"] = {str(g): round(t, 3) for g, t in times.items()}
            self.save()
        return int(ent["near_grid"])

    def width(self, prob: BorGpuProblem, nrhs: int) -> int:
        """Class width for bodies of this size bucket: the candidate whose padded
        LU + substitutions (measured on one mode system of this size, scaled by
        the body's modes) cost least, the padding included."""
        torch = prob.torch
        k = self.key(torch.cuda.get_device_name(prob.device), prob.n, prob.n_xi, prob.m_max)
        ent = self.table.setdefault(k, {})
        if "width" not in ent:
            lib = nat.load()
            st = nat.stream_handle()
            cost = {}
            for w in self.WIDTHS:
                n_pad = -(-prob.n // w) * w
                batch = min(prob.m_max + 1, 8)
                A = torch.randn((batch, n_pad, n_pad), dtype=torch.complex64, device=prob.device)
                A += n_pad * torch.eye(n_pad, dtype=torch.complex64, device=prob.device)
                B = torch.randn((batch, n_pad, nrhs), dtype=torch.complex64, device=prob.device)
                ipiv = torch.empty((batch, n_pad), dtype=torch.int32, device=prob.device)
                info = torch.empty((batch,), dtype=torch.int32, device=prob.device)
                lw = torch.empty(int(lib.ghost_bor_getrf_workspace(nat.F32, batch, n_pad)), dtype=torch.uint8,
                                 device=prob.device)
                rw = torch.empty(int(lib.ghost_bor_getrs_workspace(nat.F32, batch, n_pad, nrhs)),
                                 dtype=torch.uint8, device=prob.device)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                A0 = A.clone()
                for rep in range(2):                       # the first run warms up
                    A.copy_(A0)
                    e0.record()
                    nat.call("ghost_bor_getrf", nat.F32, batch, n_pad, nat.ptr(A), n_pad, A.stride(0),
                             nat.ptr(ipiv), nat.ptr(info), nat.ptr(lw), st)
                    nat.call("ghost_bor_getrs", nat.F32, batch, n_pad, nrhs, nat.ptr(A), n_pad, A.stride(0),
                             nat.ptr(ipiv), nat.ptr(B), nrhs, B.stride(0), nat.ptr(rw), st)
                    e1.record()
                torch.cuda.synchronize()
                cost[w] = e0.elapsed_time(e1) / batch
                del A, A0, B, lw, rw
            # the measured cost includes this body's padding; a wider class also
            # groups more bodies into one batch, which the measurement on one body
            # cannot see: credit it by the square root of the width ratio
            score = {w: cost[w] / math.sqrt(w / self.WIDTHS[0]) for w in self.WIDTHS}
            ent["width"] = min(score, key=score.get)
            ent["lu_ms_per_mode"] = {str(w): round(c, 4) for w, c in cost.items()}
            self.save()
        return int(ent["width"])


# ---------------------------------------------------------------------------
# size classes
# ---------------------------------------------------------------------------
@dataclass
class _Member:
    index: int
    prob: BorGpuProblem
    off: int                   # first mode of this body in the class arrays
    band: object = None
    rhs_ws: object = None
    ex_chunk: int = 1


@dataclass
class _Class:
    n_pad: int
    members: List[_Member]
    T: int                     # modes of all members
    bufs: Dict[str, object] = field(default_factory=dict)
    graph: object = None
    near_grid: int = 0         # near-fill CTAs per SM (0: the library default)
    launches: int = 0          # library launches of one sweep (captured in the graph)
    up_chunk: int = 1


def _class_bytes(T: int, n: int, nrhs: int) -> int:
    # Zf (c128), A and Ac (c64); B, X, R64 (c128); X32, R32 (c64)
    return T * n * n * 32 + T * n * nrhs * 64


class BorGpuBatch:
    """Monostatic sweeps of many bodies (same angles, EFIE, PEC) as size classes."""

    WS_BYTES = 4 << 30          # bound of one GEMM-update / exact-residual scratch

    def __init__(self, problems: Sequence[BorGpuProblem], tuner: Optional[Autotuner] = None,
                 width: Optional[int] = None, mem_fraction: float = 0.5, max_refine: int = 3):
        probs = list(problems)
        if not probs:
            raise ValueError("no bodies")
        p0 = probs[0]
        for p in probs:
            if p.alpha != 1.0:
                raise NotImplementedError("the batched sweep covers the EFIE formulation")
            if p.T != p0.T or not np.array_equal(p.thetas, p0.thetas):
                raise ValueError("every body of a batch must use the same aspect angles")
        self.torch = p0.torch
        self.device = p0.device
        self.nrhs = p0.nrhs
        self.max_refine = max_refine
        self.tuner = tuner
        torch = self.torch
        free, _ = torch.cuda.mem_get_info(self.device)
        # blocks cached by torch's allocator are free for the batch too
        free += torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
        budget = mem_fraction * free
        self.budget = budget
        order = sorted(range(len(probs)), key=lambda i: probs[i].n)
        self.classes: List[_Class] = []
        cur: List[int] = []
        cur_pad = 0
        for i in order:
            p = probs[i]
            w = width or (tuner.width(p, self.nrhs) if tuner else 256)
            n_pad = -(-p.n // w) * w
            T_new = sum(probs[j].m_max + 1 for j in cur) + p.m_max + 1
            if cur and (n_pad != cur_pad or _class_bytes(T_new, n_pad, self.nrhs) > budget):
                self._add_class(probs, cur, cur_pad)
                cur = []
            if not cur:
                cur_pad = n_pad
            cur.append(i)
        if cur:
            self._add_class(probs, cur, cur_pad)
        self.n_bodies = len(probs)

    def _add_class(self, probs, idx, n_pad):
        members, off = [], 0
        for i in idx:
            members.append(_Member(i, probs[i], off))
            off += probs[i].m_max + 1
        c = _Class(n_pad, members, off)
        if self.tuner is not None:
            c.near_grid = self.tuner.near_grid(members[0].prob)
        self.classes.append(c)

    # -- buffers ------------------------------------------------------------
    def _alloc(self, c: _Class):
        torch = self.torch
        lib = nat.load()
        dev = self.device
        T, n, nrhs = c.T, c.n_pad, self.nrhs
        c128, c64 = torch.complex128, torch.complex64
        b = c.bufs
        b["Zf"] = torch.zeros((T, n, n), dtype=c128, device=dev)
        b["A"] = torch.zeros((T, n, n), dtype=c64, device=dev)
        b["Ac"] = torch.zeros((T, n, n), dtype=c64, device=dev)
        b["B"] = torch.zeros((T, n, nrhs), dtype=c128, device=dev)
        b["X"] = torch.zeros((T, n, nrhs), dtype=c128, device=dev)
        b["R64"] = torch.zeros((T, n, nrhs), dtype=c128, device=dev)
        b["X32"] = torch.zeros((T, n, nrhs), dtype=c64, device=dev)
        b["R32"] = torch.zeros((T, n, nrhs), dtype=c64, device=dev)
        b["norms"] = torch.zeros((T, 2), dtype=torch.float64, device=dev)
        b["bnorm"] = torch.zeros((T,), dtype=torch.float64, device=dev)
        b["ipiv"] = torch.zeros((T, n), dtype=torch.int32, device=dev)
        b["info"] = torch.zeros((T,), dtype=torch.int32, device=dev)
        b["dF"] = torch.zeros((T, nrhs), dtype=c128, device=dev)
        b["lu_ws"] = torch.empty(int(lib.ghost_bor_getrf_workspace(nat.F32, T, n)), dtype=torch.uint8, device=dev)
        b["rs_ws"] = torch.empty(int(lib.ghost_bor_getrs_workspace(nat.F32, T, n, nrhs)), dtype=torch.uint8,
                                 device=dev)
        # scratch of the GEMM updates and of the exact residual, in mode chunks
        # bounded by WS_BYTES (as the single-body sweep)
        per = int(lib.ghost_bor_cgemm_tc_workspace(1, n, nrhs, n))
        c.up_chunk = max(1, min(T, int(self.WS_BYTES // max(per, 1))))
        b["up_ws"] = torch.empty(int(lib.ghost_bor_cgemm_tc_workspace(c.up_chunk, n, nrhs, n)),
                                 dtype=torch.uint8, device=dev)
        n_up = -(-T // c.up_chunk)
        b["up_status"] = torch.zeros((max(1, self.max_refine) * n_up,), dtype=torch.int32, device=dev)
        ex_bytes = 0
        for m in c.members:
            per = int(lib.ghost_bor_residual_exact_workspace(1, m.prob.n, nrhs))
            m.ex_chunk = max(1, min(m.prob.m_max + 1, int(self.WS_BYTES // max(per, 1))))
            ex_bytes = max(ex_bytes, int(lib.ghost_bor_residual_exact_workspace(m.ex_chunk, m.prob.n, nrhs)))
        b["ex_ws"] = torch.empty(ex_bytes, dtype=torch.uint8, device=dev)
        b["ex_flags"] = torch.zeros((len(c.members),), dtype=torch.int32, device=dev)
        for m in c.members:
            p = m.prob
            m.band = torch.zeros((p.m_max + 1, 4, p.Nn, 5), dtype=c128, device=dev)
            m.rhs_ws = torch.empty(int(lib.ghost_bor_rhs_workspace(p.N, p.m_max, p.T)), dtype=torch.uint8,
                                   device=dev)
        # identity in the padded rows / columns of every mode system; B's padded
        # rows stay zero (nothing writes them), so the padded unknowns are zero
        pads = {}
        for m in c.members:
            if m.prob.n < n:
                pads.setdefault(m.prob.n, []).append((m.off, m.off + m.prob.m_max + 1))
        b["pads"] = list(pads.items())

    # -- one sweep of a class (stream-ordered, no host synchronisation) -----
    def _run(self, c: _Class):
        torch = self.torch
        b = c.bufs
        st = nat.stream_handle()
        T, n, nrhs = c.T, c.n_pad, self.nrhs
        Zf, A, Ac, B, X, R64, X32, R32 = (b[k] for k in ("Zf", "A", "Ac", "B", "X", "R64", "X32", "R32"))
        norms = b["norms"]
        l0 = nat.launch_count()
        Zf.zero_()
        for m in c.members:
            p, o, Mb = m.prob, m.off, m.prob.m_max + 1
            Zi = Zf[o:o + Mb]
            p.fill_operator_far(Zi, nat.F32, st)
            m.band.zero_()
            p.fill_operator_near(st, band=m.band, precision=nat.F32)
            for dst in (A, Ac):
                nat.call("ghost_bor_compose", Mb, p.n, p.Nn, nat.ptr(Zi), n, Zf.stride(0), nat.ptr(m.band),
                         nat.ptr(p.d_masks), nat.ptr(dst[o]), n, dst.stride(0), st)
            nat.call("ghost_bor_rhs", p.N, p.m_max, p.T, p.k, 1.0, 0.0, nat.ptr(p.d_geo), nat.ptr(p.d_thetas),
                     nat.ptr(p.d_masks), nat.ptr(B[o]), nrhs, B.stride(0), nat.ptr(m.rhs_ws), st)
        for ni, spans in b["pads"]:
            for o0, o1 in spans:
                for dst in (A, Ac):
                    dst[o0:o1, ni:, :].zero_()
                    dst[o0:o1, :ni, ni:].zero_()
                    dst[o0:o1, ni:, ni:].diagonal(dim1=-2, dim2=-1).fill_(1.0)
        nat.call("ghost_bor_convert", 0, T, n, nrhs, nat.ptr(B), nrhs, B.stride(0), nat.ptr(X32), nrhs,
                 X32.stride(0), st)
        nat.call("ghost_bor_getrf", nat.F32, T, n, nat.ptr(A), n, A.stride(0), nat.ptr(b["ipiv"]),
                 nat.ptr(b["info"]), nat.ptr(b["lu_ws"]), st)
        nat.call("ghost_bor_getrs", nat.F32, T, n, nrhs, nat.ptr(A), n, A.stride(0), nat.ptr(b["ipiv"]),
                 nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(b["rs_ws"]), st)
        nat.call("ghost_bor_convert", 1, T, n, nrhs, nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(X), nrhs,
                 X.stride(0), st)

        def exact(Xin, Bin, first):
            for j, m in enumerate(c.members):
                p, Mb = m.prob, m.prob.m_max + 1
                for q0 in range(0, Mb, m.ex_chunk):
                    nb, o = min(m.ex_chunk, Mb - q0), m.off + q0
                    nat.call("ghost_bor_residual_exact", nb, p.n, nrhs, p.Nn, nat.ptr(Zf[o]), n, Zf.stride(0),
                             nat.ptr(m.band[q0]), nat.ptr(p.d_masks[q0]), nat.ptr(Xin[o]), nat.ptr(Bin[o]), nrhs,
                             Bin.stride(0), nat.ptr(R64[o]), nat.ptr(R32[o]), nat.ptr(norms[o]),
                             nat.ptr(b["ex_ws"]), b["ex_ws"].numel(), st)
                    torch.maximum(b["ex_flags"][j:j + 1], b["ex_ws"][:4].view(torch.int32),
                                  out=b["ex_flags"][j:j + 1])
            if first:
                b["bnorm"].copy_(norms[:, 1])

        exact(X32, B, True)
        for it in range(self.max_refine):
            nat.call("ghost_bor_convert", 3, T, n, nrhs, nat.ptr(R32), nrhs, R32.stride(0), nat.ptr(X32), nrhs,
                     X32.stride(0), st)
            nat.call("ghost_bor_getrs", nat.F32, T, n, nrhs, nat.ptr(A), n, A.stride(0), nat.ptr(b["ipiv"]),
                     nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(b["rs_ws"]), st)
            nat.call("ghost_bor_convert", 2, T, n, nrhs, nat.ptr(X32), nrhs, X32.stride(0), nat.ptr(X), nrhs,
                     X.stride(0), st)
            if it == 0:
                exact(X32, R64, False)                 # R -= Z D with exact products
            else:
                n_up = -(-T // c.up_chunk)
                for ci, q0 in enumerate(range(0, T, c.up_chunk)):
                    nb = min(c.up_chunk, T - q0)
                    nat.call("ghost_bor_cgemm_tc", nb, n, nrhs, n, nat.ptr(Ac[q0]), n, Ac.stride(0),
                             nat.ptr(X32[q0]), nrhs, X32.stride(0), nat.ptr(R32[q0]), nrhs, R32.stride(0),
                             nat.ptr(b["up_ws"]), nat.ptr(b["up_status"][it * n_up + ci]), st)
        # residual of the last correction's update, relative to ||B||, per mode
        rn = torch.linalg.vector_norm(R32, dim=(1, 2)).double() ** 2
        norms[:, 0].copy_(rn)
        for m in c.members:
            p, o, Mb = m.prob, m.off, m.prob.m_max + 1
            nat.call("ghost_bor_farfield", nat.F64, Mb, p.n, nrhs, p.Nn, p.k, nat.ptr(p.d_mode_w), nat.ptr(B[o]),
                     nrhs, B.stride(0), nat.ptr(X[o]), nrhs, X.stride(0), nat.ptr(b["dF"][o]), st)
        return nat.launch_count() - l0

    # -- public -------------------------------------------------------------
    def resident(self) -> bool:
        """Whether every class's buffers fit the memory budget at once (then
        they stay allocated between sweeps and the classes replay as graphs)."""
        return sum(_class_bytes(c.T, c.n_pad, self.nrhs) for c in self.classes) <= self.budget

    def sweep(self, use_graphs: bool = True) -> List[SweepResult]:
        """FP32 + FP64-refinement sweep of every body; returns one SweepResult
        per body in the order given.

        Resident batches (all classes fit the budget): the first call allocates
        each class's buffers, runs it once and (use_graphs) captures it as a CUDA
        graph; later calls replay the graphs.  Larger batches stream: each class
        is allocated, swept (eagerly, still without host synchronisation inside)
        and released before the next."""
        torch = self.torch
        out: List[Optional[SweepResult]] = [None] * self.n_bodies
        lib = nat.load()
        keep = self.resident()
        for c in self.classes:
            if not c.bufs:
                self._alloc(c)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            if not keep:
                lib.ghost_bor_set_near_grid(c.near_grid)
                try:
                    e0.record()
                    c.launches = self._run(c)
                    e1.record()
                finally:
                    lib.ghost_bor_set_near_grid(0)
            elif c.graph is None:
                lib.ghost_bor_set_near_grid(c.near_grid)
                try:
                    e0.record()
                    c.launches = self._run(c)
                    e1.record()
                    if use_graphs:
                        torch.cuda.synchronize()
                        g = torch.cuda.CUDAGraph()
                        with torch.cuda.graph(g):
                            self._run(c)
                        c.graph = g
                finally:
                    lib.ghost_bor_set_near_grid(0)
            else:
                e0.record()
                c.graph.replay()
                e1.record()
            torch.cuda.synchronize()
            self._check(c)
            secs = e0.elapsed_time(e1) / 1e3
            b = c.bufs
            dF = b["dF"].cpu().numpy()
            res = torch.sqrt(b["norms"][:, 0] / torch.clamp(b["bnorm"], min=1e-300)).cpu().numpy()
            info = b["info"].cpu().numpy()
            for m in c.members:
                p, o, Mb = m.prob, m.off, m.prob.m_max + 1
                d = dF[o:o + Mb].reshape(Mb, p.T, 2).transpose(0, 2, 1)
                out[m.index] = SweepResult(
                    dF=np.ascontiguousarray(d), residual=res[o:o + Mb], refine_iters=self.max_refine,
                    timings={"class_gpu_s": secs, "class_bodies": len(c.members), "class_n_pad": c.n_pad,
                             "graph": c.graph is not None},
                    info=info[o:o + Mb], gpu_launches=c.launches)
            if not keep:
                c.bufs.clear()
                for m in c.members:
                    m.band = m.rhs_ws = None
        return out

    def _check(self, c: _Class):
        b = c.bufs
        for m in c.members:
            m.prob.check_near_status()
            m.prob.check_far_status()
        if int(b["ex_flags"].max()) != 0 or int(b["up_status"].max()) != 0 or int(b["lu_ws"][:4].view(
                self.torch.int32)[0]) != 0 or int(b["rs_ws"][:4].view(self.torch.int32)[0]) != 0:
            raise RuntimeError("a bounded tensor-core wait gave up in a batched sweep")

    def summary(self) -> List[Dict]:
        return [{"n_pad": c.n_pad, "bodies": len(c.members), "modes": c.T,
                 "n": [m.prob.n for m in c.members]} for c in self.classes]
