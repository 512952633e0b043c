"""Recorded forest steps (CUDA graph): a replayed step must give exactly the results of the
ordinary calls on the same inputs, also after the entities and queries were changed in place."""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import assert_csr_equal

pytestmark = pytest.mark.gpu


def _data(rng, sizes):
    n = int(sizes.sum())
    c = rng.random((n, 3)) * 100
    e = rng.uniform(0.05, 1.0, (n, 3))
    ent = np.concatenate([c - e, c + e], 1).astype(np.float32)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    t = len(sizes)
    qc = rng.random((t * 64, 3)) * 100
    qe = rng.uniform(0.5, 5, (t * 64, 3))
    ranges = np.concatenate([qc - qe / 2, qc + qe / 2], 1).astype(np.float32)
    d = rng.normal(size=(t * 64, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([rng.random((t * 64, 3)) * 100, d], 1).astype(np.float32)
    planes = np.zeros((t, 6, 4), np.float32)
    for i in range(t):
        lo, hi = rng.random(3) * 40, 60 + rng.random(3) * 40
        for a in range(3):
            planes[i, 2 * a, 0], planes[i, 2 * a, 1 + a] = lo[a], 1.0
            planes[i, 2 * a + 1, 0], planes[i, 2 * a + 1, 1 + a] = -hi[a], -1.0
    return ent, off, ranges, rays, planes


def _reference(ent, off, ranges, rays, planes, qoff, foff):
    f = otg.Forest("boxes", np.float32).create(ent, off, max_elements=16)
    return f.range_search(ranges, qoff), f.ray_all(rays, qoff), f.frustum_culling(planes, foff)


def test_plan_replays_match_ordinary_calls():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(121)
    sizes = rng.integers(1000, 20000, 32)
    ent, off, ranges, rays, planes = _data(rng, sizes)
    qoff = np.arange(33, dtype=np.uint64) * 64
    foff = np.arange(33, dtype=np.uint64)
    d_ent, d_r, d_y, d_p = (torch.as_tensor(x, device="cuda") for x in (ent, ranges, rays, planes))
    forest = otg.Forest("boxes", np.float32)
    plan = otg.ForestPlan(forest, d_ent, off, max_elements=16, ranges=d_r, range_offsets=qoff, rays=d_y, ray_offsets=qoff, planes=d_p,
                          frustum_offsets=foff, capacity_factor=2.0)
    for step in range(3):
        if step:
            shift = torch.as_tensor(rng.normal(0, 0.3, (len(ent), 3)).astype(np.float32), device="cuda")
            d_ent += torch.cat([shift, shift], 1)
            d_r += 0.25
        plan.run()
        want = _reference(d_ent.cpu().numpy(), off, d_r.cpu().numpy(), rays, planes, qoff, foff)
        got = [plan.result(k) for k in range(3)]
        assert_csr_equal(got[0][:2], want[0][:2], f"step {step} range")
        assert_csr_equal(got[1], want[1], f"step {step} ray_all")
        assert_csr_equal(got[2][:2], want[2][:2], f"step {step} frustum")


def test_plan_reports_capacity_overflow():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(122)
    sizes = rng.integers(1000, 5000, 8)
    ent, off, ranges, rays, planes = _data(rng, sizes)
    qoff = np.arange(9, dtype=np.uint64) * 64
    d_ent, d_r = torch.as_tensor(ent, device="cuda"), torch.as_tensor(ranges, device="cuda")
    plan = otg.ForestPlan(otg.Forest("boxes", np.float32), d_ent, off, max_elements=16, ranges=d_r, range_offsets=qoff, capacity_factor=1.0)
    plan.run()
    plan.result(0)
    # every range now covers the whole space: far more ids than the capacity recorded
    d_r[:, :3] = -10.0
    d_r[:, 3:] = 110.0
    plan.run()
    with pytest.raises(otg.OtgError):
        plan.result(0)
