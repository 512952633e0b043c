"""The batched FP32-filtered kNN (warp per query, FP64 recheck) against the CPU oracle and against the
plain one-query-per-thread FP64 kernel: ids and distances bit-exact, for uneven k, bounded search
distances, ties, k = 0 (an empty result, as in the reference), the filter's fallback cases (k above the
buffer limit, candidate overflow)
and both scalar types. The recheck fraction must stay small on random data."""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import assert_csr_equal
from _oracle_lib import KIND_POINTS, oracle

pytestmark = pytest.mark.gpu


def _mixture(n, seed, dtype=np.float64):
    rng = np.random.default_rng(seed)
    m = int(n * 0.3)
    u = rng.random((n - m, 3))
    d = rng.normal(size=(m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    s = 0.5 + d * rng.normal(0.4, 0.005, (m, 1))
    pts = np.concatenate([u, s])
    rng.shuffle(pts)
    return pts.astype(dtype)


def _both(t, q, k, **kw):
    f = t.knn(q, k, algo=otg.ALGO_FILTERED, **kw)
    p = t.knn(q, k, algo=otg.ALGO_PLAIN_FP64, **kw)
    return f, p


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_filtered_uneven_k_matches_oracle_and_plain(dtype):
    pts = _mixture(300_000, 61, dtype)
    q = _mixture(4000, 62, dtype)
    k = np.random.default_rng(63).integers(1, 65, len(q)).astype(np.uint32)
    t = otg.Tree("points", dtype).create(pts, max_depth=10, max_elements=20)
    o = oracle().create(pts, KIND_POINTS, 10, None, 20)
    f, p = _both(t, q, k)
    assert_csr_equal(f, p, "filtered vs plain")
    assert_csr_equal(f, o.knn(q, k), "filtered vs oracle")


def test_filtered_recheck_fraction_is_small():
    pts = _mixture(300_000, 64)
    q = _mixture(4000, 65)
    t = otg.Tree("points").create(pts, max_depth=10, max_elements=20)
    r = t.knn(q, 16, algo=otg.ALGO_FILTERED, raw=True)
    tests, rechecks = r.stats()
    assert tests > 0 and rechecks >= 16 * len(q)
    assert rechecks / tests < 0.5, (tests, rechecks)


@pytest.mark.parametrize("k", [0, 1, 150, 240, 241, 256])
def test_filtered_k_range_and_fallbacks(k):
    pts = _mixture(50_000, 66)
    q = _mixture(500, 67)
    t = otg.Tree("points").create(pts, max_depth=8, max_elements=16)
    o = oracle().create(pts, KIND_POINTS, 8, None, 16)
    if k == 0:
        f, p = _both(t, q, k, max_distance=0.02)
        assert_csr_equal(f, p, "k=0 filtered vs plain")
        assert_csr_equal(f, o.knn(q, k, max_dist=0.02), "k=0 vs oracle")
        return
    f, p = _both(t, q, k)
    assert_csr_equal(f, p, f"k={k} filtered vs plain")
    assert_csr_equal(f, o.knn(q, k), f"k={k} vs oracle")


@pytest.mark.parametrize("md", [0.0, 1e-3, 0.05, 3.0])
def test_filtered_max_distance(md):
    pts = _mixture(100_000, 68)
    q = np.concatenate([_mixture(500, 69), np.array([[5.0, 5.0, 5.0], [-3.0, 0.5, 0.5]])])
    t = otg.Tree("points").create(pts, max_depth=9, max_elements=20)
    o = oracle().create(pts, KIND_POINTS, 9, None, 20)
    f, p = _both(t, q, 12, max_distance=md)
    assert_csr_equal(f, p, f"maxdist {md} filtered vs plain")
    assert_csr_equal(f, o.knn(q, 12, max_dist=md), f"maxdist {md} vs oracle")


def test_filtered_ties_and_duplicates():
    rng = np.random.default_rng(70)
    lattice = np.round(rng.random((30_000, 3)) * 30)  # exact ties in every query's neighbourhood
    dup = np.tile(np.array([[7.0, 7.0, 7.0]]), (1500, 1))  # candidate overflow -> plain kernels
    pts = np.concatenate([lattice, dup])
    t = otg.Tree("points").create(pts, max_depth=6, max_elements=8)
    o = oracle().create(pts, KIND_POINTS, 6, None, 8)
    q = np.concatenate([np.round(rng.random((400, 3)) * 30) + 0.5, np.round(rng.random((100, 3)) * 30), [[7.0, 7.0, 7.0], [7.2, 7.0, 7.0]]])
    for k in (1, 7, 30):
        f, p = _both(t, q, k)
        assert_csr_equal(f, p, f"ties k={k} filtered vs plain")
        assert_csr_equal(f, o.knn(q, k), f"ties k={k} vs oracle")


def test_filtered_given_box_and_outside_points():
    rng = np.random.default_rng(71)
    pts = rng.random((60_000, 3)) * 10 - 5
    pts[:50] *= 3  # outside the given box: kept at the root
    box = np.array([-5.0, -5.0, -5.0, 5.0, 5.0, 5.0])
    t = otg.Tree("points").create(pts, max_depth=7, box=box, max_elements=12)
    o = oracle().create(pts, KIND_POINTS, 7, box, 12)
    q = rng.random((600, 3)) * 24 - 12
    f, p = _both(t, q, 9)
    assert_csr_equal(f, p, "outside filtered vs plain")
    assert_csr_equal(f, o.knn(q, 9), "outside vs oracle")


def test_filtered_device_inputs_and_rebuild():
    torch = pytest.importorskip("torch")
    pts = _mixture(80_000, 72)
    q = _mixture(2000, 73)
    k = np.random.default_rng(74).integers(1, 40, len(q)).astype(np.uint32)
    t = otg.Tree("points").create(torch.as_tensor(pts, device="cuda"), max_depth=9, max_elements=20)
    a = t.knn(torch.as_tensor(q, device="cuda"), torch.as_tensor(k.astype(np.int32), device="cuda"))
    o = oracle().create(pts, KIND_POINTS, 9, None, 20)
    assert_csr_equal(a, o.knn(q, k), "device inputs")
    # a rebuild must refresh the FP32 image
    pts2 = _mixture(80_000, 75)
    t.create(pts2, max_depth=9, max_elements=20)
    o2 = oracle().create(pts2, KIND_POINTS, 9, None, 20)
    assert_csr_equal(t.knn(q, k), o2.knn(q, k), "after rebuild")


@pytest.mark.parametrize("layout", ["far_offset", "near_ties"])
def test_filtered_margin_at_large_coordinates(layout):
    """The FP32 filter's margins where an FP32 ulp approaches the gap at the k-th distance: FP64
    trees at coordinates around 1e6-1e7 (an FP32 ulp there is 0.06-1), and (near_ties) query points
    whose neighbours lie at distances differing by about one FP32 ulp of the coordinates. Filtered,
    plain and oracle agree id for id and distance for distance. (FP32 trees at such coordinates
    store them on a grid of 0.25-1, so exact ties at the k-th distance bound are common, where the
    reference's own result depends on its traversal order.)"""
    dtype = np.float64
    rng = np.random.default_rng(91)
    n = 200_000
    if layout == "far_offset":
        # a cube of side 100 placed at 2.5e6 .. 7.5e6 + 100, points on a 1/16 lattice with jitter
        # (many near-equal distances)
        base = np.array([5.0e6, 7.5e6, 2.5e6])
        pts = base + np.round(rng.random((n, 3)) * 1600) / 16 + rng.normal(0, 1e-3, (n, 3))
        q = base + rng.random((2000, 3)) * 100
    else:
        # per query, 100 points at radius 3 +- up to one FP32 ulp of 8e6 around it
        base = 8.0e6
        c = base + rng.random((2000, 3)) * 1000
        dirs = rng.normal(size=(2000, 100, 3))
        dirs /= np.linalg.norm(dirs, axis=2, keepdims=True)
        r = 3.0 + rng.integers(-2, 3, (2000, 100, 1)) * float(np.spacing(np.float32(base))) * 0.5
        pts = (c[:, None, :] + dirs * r).reshape(-1, 3)
        q = c
    pts = pts.astype(dtype)
    q = q.astype(dtype)
    k = np.random.default_rng(92).integers(1, 33, len(q)).astype(np.uint32)
    t = otg.Tree("points", dtype).create(pts, max_depth=10, max_elements=20)
    o = oracle().create(pts, KIND_POINTS, 10, None, 20)
    f, p = _both(t, q, k)
    ref = o.knn(q, k)
    assert_csr_equal(p, ref, "plain vs oracle")
    assert_csr_equal(f, ref, "filtered vs oracle")
