"""The FP32-filtered collision search (packets of 32 boxes, outward-rounded FP32 images, exact
recheck of undecided pairs) against the plain FP64 kernel and the CPU oracle: pair lists identical,
within one tree and between two trees, for clustered boxes, touching boxes at the tolerance,
degenerate boxes and both scalar types."""
import numpy as np
import pytest

import octree_gb300 as otg
from _oracle_lib import KIND_LOOSE_BOXES, oracle

pytestmark = pytest.mark.gpu


def _clustered(n, seed, span=100.0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    half = n // 2
    c = np.empty((n, 3))
    c[:half] = rng.random((half, 3)) * span
    cc = rng.random((16, 3)) * span
    c[half:] = cc[rng.integers(0, 16, n - half)] + rng.normal(0, span / 100, (n - half, 3))
    ext = rng.lognormal(np.log(span / 2000), 0.6, (n, 3))
    return np.concatenate([c - ext, c + ext], 1).astype(dtype)


def _pairs(t, algo, other=None):
    return t.collision_self(algo=algo) if other is None else t.collision_pair(other, algo=algo)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_filtered_self_collision(dtype):
    boxes = _clustered(60_000, 81, dtype=dtype)
    t = otg.Tree("boxes", dtype).create(boxes, max_depth=8, max_elements=32)
    f = _pairs(t, otg.ALGO_FILTERED)
    p = _pairs(t, otg.ALGO_PLAIN_FP64)
    assert len(f) > 1000
    assert np.array_equal(f, p)
    o = oracle().create(boxes, KIND_LOOSE_BOXES, 8, None, 32)
    assert np.array_equal(f, o.collide_self())
    r = t.collision_self(algo=otg.ALGO_FILTERED, raw=True)
    tests, rechecks = r.stats()
    assert tests > 0 and rechecks < tests * 0.05


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_filtered_pair_collision(dtype):
    a = _clustered(40_000, 82, dtype=dtype)
    rng = np.random.default_rng(83)
    b = (a[:30_000].astype(np.float64) + rng.normal(0, 0.05, (30_000, 1))).astype(dtype)  # moved copies: many pairs
    ta = otg.Tree("boxes", dtype).create(a, max_depth=8, max_elements=24)
    tb = otg.Tree("boxes", dtype).create(b, max_depth=7, max_elements=16)
    f = _pairs(ta, otg.ALGO_FILTERED, tb)
    p = _pairs(ta, otg.ALGO_PLAIN_FP64, tb)
    assert len(f) > 100
    assert np.array_equal(f, p)
    oa = oracle().create(a, KIND_LOOSE_BOXES, 8, None, 24)
    ob = oracle().create(b, KIND_LOOSE_BOXES, 7, None, 16)
    assert np.array_equal(f, oa.collide_pair(ob))


def test_filtered_touching_and_degenerate_boxes():
    rng = np.random.default_rng(84)
    # unit lattice boxes: neighbours touch exactly (adjacent, not overlapping), plus boxes that
    # overlap their neighbours by less than, exactly and more than the tolerance
    g = np.stack(np.meshgrid(np.arange(12), np.arange(12), np.arange(12), indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    lattice = np.concatenate([g, g + 1.0], 1)
    tol = 2.220446049250313e-14
    shifted = lattice[:300].copy()
    shifted[:100, 3] += tol * 0.5
    shifted[100:200, 3] += tol
    shifted[200:300, 3] += tol * 4
    flat = np.concatenate([g[:200] + 0.5, g[:200] + 0.5], 1)  # zero-size boxes
    flat[:, 3] += rng.random(200)
    boxes = np.concatenate([lattice, shifted, flat])
    t = otg.Tree("boxes").create(boxes, max_depth=5, max_elements=8)
    f = _pairs(t, otg.ALGO_FILTERED)
    p = _pairs(t, otg.ALGO_PLAIN_FP64)
    assert np.array_equal(f, p)
    o = oracle().create(boxes, KIND_LOOSE_BOXES, 5, None, 8)
    assert np.array_equal(f, o.collide_self())


def test_filtered_far_coordinates_float():
    # float trees with coordinates far above the tolerance: the rounding-gap cases of GetBoxRelation
    rng = np.random.default_rng(85)
    c = rng.random((20_000, 3)) * 64 + 128
    e = rng.random((20_000, 3)) * 0.05
    boxes = np.concatenate([c - e, c + e], 1).astype(np.float32)
    # partners one ulp (more than the tolerance, less than its rounding) beyond each box in x
    gap = boxes[:2000].copy()
    width = gap[:, 3] - gap[:, 0]
    gap[:, 0] = np.nextafter(boxes[:2000, 3], np.float32(np.inf))
    gap[:, 3] = gap[:, 0] + width
    boxes = np.concatenate([boxes, gap])
    t = otg.Tree("boxes", np.float32).create(boxes, max_depth=7, max_elements=16)
    f = _pairs(t, otg.ALGO_FILTERED)
    p = _pairs(t, otg.ALGO_PLAIN_FP64)
    assert np.array_equal(f, p)
    o = oracle().create(boxes, KIND_LOOSE_BOXES, 7, None, 16)
    assert np.array_equal(f, o.collide_self())
