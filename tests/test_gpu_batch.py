"""Batched sweeps of many bodies (batch.BorGpuBatch): size classes with padded
identity rows, one LU / substitution / refinement for all modes of a class,
CUDA-graph capture and replay, and the autotuner's JSON cache."""
import json
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bodies(pkg):
    rng = np.random.default_rng(5)
    out = []
    for n in (40, 56, 61, 90, 130):
        pts, arclen, _ = pkg.bodies.random_body(rng, n)
        k = 2.0 * math.pi * n / (16.0 * arclen)
        out.append((pts, k * 299792458.0 / (2 * math.pi), int(math.ceil(k * pts[:, 0].max())) + 6))
    return out


def _problems(pkg, bodies, thetas):
    return [pkg.engine.BorGpuProblem(p, f, thetas, m_max=m) for p, f, m in bodies]


def test_batch_matches_single_body_sweeps(pkg, bodies, tmp_path):
    batch_mod = pkg.batch
    thetas = np.arange(0.0, 181.0, 5.0)
    probs = _problems(pkg, bodies, thetas)
    tuner = batch_mod.Autotuner(str(tmp_path / "autotune.json"))
    B = batch_mod.BorGpuBatch(probs, tuner=tuner, width=128)
    assert len(B.classes) < len(probs)            # bodies share classes
    assert B.resident()
    first = B.sweep(use_graphs=True)              # eager run + capture
    again = B.sweep(use_graphs=True)              # graph replay
    assert all(r.timings["graph"] for r in again)
    for p, r1, r2 in zip(probs, first, again):
        ref64 = p.sweep("fp64").dF.sum(0)
        single = p.sweep("fp32ir").dF.sum(0)
        for r in (r1, r2):
            F = r.dF.sum(0)
            assert np.max(np.abs(F - ref64)) < 1e-6 * np.max(np.abs(ref64))
            assert np.max(np.abs(F - single)) < 1e-6 * np.max(np.abs(ref64))
            assert np.all(r.info == 0)
        np.testing.assert_allclose(r2.dF, r1.dF, rtol=0, atol=1e-12 * np.max(np.abs(r1.dF)))
    table = json.load(open(tmp_path / "autotune.json"))
    assert table and all("near_grid" in v for v in table.values())


def test_batch_streams_when_over_budget(pkg, bodies):
    thetas = np.arange(0.0, 181.0, 10.0)
    probs = _problems(pkg, bodies[:3], thetas)
    B = pkg.batch.BorGpuBatch(probs, width=128)
    B.budget = 1.0                                # force streaming: classes allocated and released in turn
    out = B.sweep()
    assert not B.resident() and all(not c.bufs for c in B.classes)
    for p, r in zip(probs, out):
        ref64 = p.sweep("fp64").dF.sum(0)
        assert np.max(np.abs(r.dF.sum(0) - ref64)) < 1e-6 * np.max(np.abs(ref64))
