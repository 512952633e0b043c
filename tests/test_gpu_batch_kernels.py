"""The batched warp-per-query kernels (default algorithm) against the one-query-per-thread kernels
(OTG_ALGO_PLAIN_FP64) for RangeSearch, FrustumCulling, RayIntersectedAll and PickSearch: identical id lists and
ray distances, on point and box trees of both scalar types and on a forest. Batches of at most
8192 queries run split by default (top levels per query, then their depth-2 subtrees as separate work items);
larger ones run whole, and both sizes are covered. (Both kernels are checked against the oracle by
the parity tests; this pins them to each other on larger inputs.)"""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import assert_csr_equal

pytestmark = pytest.mark.gpu


def _inputs(rng, n_q, dtype, span=100.0):
    c = rng.random((n_q, 3)) * span
    e = rng.uniform(0.5, 8, (n_q, 3))
    ranges = np.concatenate([c - e, c + e], 1).astype(dtype)
    ranges[:5] = np.array([-1, -1, -1, span + 1, span + 1, span + 1])  # root shortcut
    d = rng.normal(size=(n_q, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([rng.random((n_q, 3)) * span, d], 1).astype(dtype)
    planes = np.zeros((n_q // 8, 6, 4))
    for i in range(len(planes)):
        lo, hi = rng.random(3) * span * 0.4, span * 0.6 + rng.random(3) * span * 0.4
        for a in range(3):
            planes[i, 2 * a, 0], planes[i, 2 * a, 1 + a] = lo[a], 1.0
            planes[i, 2 * a + 1, 0], planes[i, 2 * a + 1, 1 + a] = -hi[a], -1.0
    return ranges, rays, planes.astype(dtype)


@pytest.mark.parametrize("nq", [3000, 12000])
@pytest.mark.parametrize("kind,dtype", [("points", np.float64), ("boxes", np.float64), ("boxes", np.float32), ("points", np.float32)])
def test_batch_kernels_match_plain(kind, dtype, nq):
    rng = np.random.default_rng(111)
    n = 150_000
    if kind == "points":
        ent = (rng.random((n, 3)) * 100).astype(dtype)
    else:
        c = rng.random((n, 3)) * 100
        e = rng.uniform(0.05, 1.0, (n, 3))
        ent = np.concatenate([c - e, c + e], 1).astype(dtype)
    t = otg.Tree(kind, dtype).create(ent, max_depth=8, max_elements=20)
    ranges, rays, planes = _inputs(rng, nq, dtype)
    for mode in (otg.RANGE_INSIDE, otg.RANGE_OVERLAP):
        assert_csr_equal(t.range_search(ranges, mode), t.range_search(ranges, mode, algo=otg.ALGO_PLAIN_FP64), f"range {mode}")
    assert_csr_equal(t.frustum_culling(planes)[:2], t.frustum_culling(planes, algo=otg.ALGO_PLAIN_FP64)[:2], "frustum")
    assert_csr_equal(t.ray_all(rays), t.ray_all(rays, algo=otg.ALGO_PLAIN_FP64), "ray_all")
    pts = (ent[:nq, :3] if kind == "points" else rng.random((nq, 3)) * 100).astype(dtype)  # entity points: exact hits
    assert_csr_equal(t.pick_search(pts)[:2], t.pick_search(pts, algo=otg.ALGO_PLAIN_FP64)[:2], "pick")
    assert len(t.pick_search(pts)[1]) > 0
    assert_csr_equal(t.ray_all(rays, max_distance=20.0), t.ray_all(rays, max_distance=20.0, algo=otg.ALGO_PLAIN_FP64), "ray_all bounded")


def test_batch_kernels_match_plain_on_forest():
    rng = np.random.default_rng(112)
    sizes = rng.integers(500, 30_000, 40)
    parts = []
    for s in sizes:
        c = rng.random((s, 3)) * 100
        e = rng.uniform(0.05, 1.0, (s, 3))
        parts.append(np.concatenate([c - e, c + e], 1))
    ent = np.concatenate(parts).astype(np.float32)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    f = otg.Forest("boxes", np.float32).create(ent, off, max_elements=16)
    ranges, rays, planes = _inputs(rng, 40 * 64, np.float32)
    qoff = np.arange(41, dtype=np.uint64) * 64
    poff = np.arange(41, dtype=np.uint64) * (len(planes) // 40)
    planes = planes[: 40 * (len(planes) // 40)]
    for mode in (otg.RANGE_INSIDE, otg.RANGE_OVERLAP):
        assert_csr_equal(f.range_search(ranges, qoff, mode), f.range_search(ranges, qoff, mode, algo=otg.ALGO_PLAIN_FP64), f"forest range {mode}")
    assert_csr_equal(f.frustum_culling(planes, poff)[:2], f.frustum_culling(planes, poff, algo=otg.ALGO_PLAIN_FP64)[:2], "forest frustum")
    assert_csr_equal(f.ray_all(rays, qoff), f.ray_all(rays, qoff, algo=otg.ALGO_PLAIN_FP64), "forest ray_all")


@pytest.mark.parametrize("split", [1, 2, 3, 4])
@pytest.mark.parametrize("warps", [2, 8])
def test_every_split_depth_matches_plain(warps, split):
    """Each shape the autotuner chooses among (warps per block, and no split or the subtrees at depth
    1-3 as separate work items) gives the plain kernel's results, on a point and a box tree, for a
    batch that allows every split depth and one that allows depths 1-2 only."""
    rng = np.random.default_rng(113)
    n = 120_000
    c = rng.random((n, 3)) * 100
    e = rng.uniform(0.05, 1.0, (n, 3))
    boxes = np.concatenate([c - e, c + e], 1)
    trees = [otg.Tree("points").create(c, max_depth=8, max_elements=20), otg.Tree("boxes").create(boxes, max_depth=8, max_elements=20)]
    otg.autotune_force_shape(warps | (split << 8))
    try:
        for nq in (2000, 20_000):
            ranges, rays, planes = _inputs(rng, nq, np.float64)
            for t in trees:
                ref = t.range_search(ranges, otg.RANGE_OVERLAP, algo=otg.ALGO_PLAIN_FP64)
                assert_csr_equal(t.range_search(ranges, otg.RANGE_OVERLAP), ref, f"range nq={nq}")
                assert_csr_equal(t.frustum_culling(planes)[:2], t.frustum_culling(planes, algo=otg.ALGO_PLAIN_FP64)[:2], f"frustum nq={nq}")
                assert_csr_equal(t.ray_all(rays), t.ray_all(rays, algo=otg.ALGO_PLAIN_FP64), f"ray_all nq={nq}")
    finally:
        otg.autotune_force_shape(-1)
