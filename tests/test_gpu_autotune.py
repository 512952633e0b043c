"""The kernel-shape autotuner: the first call of a size class times every shape and records its
choice; tuned, cached and untuned calls return identical results."""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import assert_csr_equal

pytestmark = pytest.mark.gpu


def test_autotuned_shapes_return_identical_results():
    rng = np.random.default_rng(131)
    pts = rng.random((200_000, 3)) * 100
    t = otg.Tree("points").create(pts, max_depth=9, max_elements=20)
    c = rng.random((3000, 3)) * 100
    ranges = np.concatenate([c - 2, c + 2], 1)
    q = rng.random((3000, 3)) * 100
    otg.autotune_enable(True)
    before = len(otg.autotune_entries())
    r1 = t.range_search(ranges)
    k1 = t.knn(q, 9)
    entries = otg.autotune_entries()
    assert len(entries) >= before + 2
    assert any(e.startswith("range") for e in entries) and any(e.startswith("knn") for e in entries)
    r2 = t.range_search(ranges)
    k2 = t.knn(q, 9)
    assert len(otg.autotune_entries()) == len(entries)  # cached, no new timing
    otg.autotune_enable(False)
    try:
        r3 = t.range_search(ranges)
        k3 = t.knn(q, 9)
    finally:
        otg.autotune_enable(True)
    r4 = t.range_search(ranges, algo=otg.ALGO_PLAIN_FP64)
    for r in (r2, r3, r4):
        assert_csr_equal(r1, r, "range")
    for k in (k2, k3):
        assert_csr_equal(k1, k, "knn")


def test_autotuned_collision():
    rng = np.random.default_rng(132)
    c = rng.random((100_000, 3)) * 100
    e = rng.uniform(0.05, 0.6, (100_000, 3))
    boxes = np.concatenate([c - e, c + e], 1)
    t = otg.Tree("boxes").create(boxes, max_depth=8, max_elements=24)
    a = t.collision_self()
    b = t.collision_self()
    assert np.array_equal(a, b)
    assert np.array_equal(a, t.collision_self(algo=otg.ALGO_PLAIN_FP64))
    assert any(e.startswith("collide self") for e in otg.autotune_entries())
