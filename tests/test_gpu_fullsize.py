"""Parity at the full sizes of the benchmark configurations: the CUDA path against the oracle on
the same seeded inputs that bench.py measures, with every id compared.

* 1M uniform points (depth 10, max 20): location keys, the node set, 10k RangeSearch boxes in both
  modes (batched and plain kernels), 10k GetNearestNeighbors with k = 8 (filtered and plain).
* 4M clustered FP64 boxes (depth 12, max 32): the node set and the whole self-collision pair list
  (filtered and plain kernels).
* 16M points, 70% uniform and 30% on a noisy shell (depth 10, max 20): location keys, the node set
  of about 3M nodes, and 20k of the 1M uneven-k kNN queries (k in 1..64; filtered and plain).

The oracle builds each tree with its location transform and sort on every host core (the same tree
as its sequential path); its queries run on host threads, one slice of the queries each."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import bench
import octree_gb300 as otg
from _compare import assert_csr_equal, assert_nodes_equal_exact
from _oracle_lib import KIND_LOOSE_BOXES, KIND_POINTS, oracle

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _par(fn, *arrays):
    """fn over `THREADS` contiguous slices of the query arrays, concatenated in query order."""
    n = len(arrays[0])
    cuts = [n * i // THREADS for i in range(THREADS + 1)]
    with ThreadPoolExecutor(THREADS) as ex:
        parts = list(ex.map(lambda i: fn(*[a[cuts[i] : cuts[i + 1]] for a in arrays]), range(THREADS)))
    return bench.concat_csr(parts)


def test_c1_uniform_1m_range_and_knn():
    pts, ranges, q = bench.c1_workload()
    t = otg.Tree("points").create(pts, max_depth=10, max_elements=20)
    o = oracle().create(pts, KIND_POINTS, 10, None, 20, threads=THREADS)
    assert t.max_depth == o.max_depth == 10
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal_exact(t.nodes(), o.nodes(), "1M points")
    for mode in (0, 1):
        ref = _par(lambda r: o.range_search(r, mode), ranges)
        assert int(ref[0][-1]) > 100_000  # about 20 hits per box
        for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
            assert_csr_equal(t.range_search(ranges, mode, algo=algo)[:2], ref, f"range mode {mode} algo {algo}")
    ref = _par(lambda x: o.knn(x, 8), q)
    for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
        assert_csr_equal(t.knn(q, 8, algo=algo), ref, f"knn k=8 algo {algo}")


def test_c2_clustered_boxes_4m_self_collision():
    boxes = bench.cluster_boxes(4_000_000, 201)
    t = otg.Tree("boxes").create(boxes, max_depth=12, max_elements=32)
    o = oracle().create(boxes, KIND_LOOSE_BOXES, 12, None, 32, threads=THREADS)
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal_exact(t.nodes(), o.nodes(), "4M boxes")
    ref = o.collide_self()
    assert len(ref) > 5_000_000  # about 9.7M pairs
    for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
        got = t.collision_self(algo=algo)
        assert got.shape == ref.shape, f"algo {algo}: {len(got)} pairs vs {len(ref)}"
        assert np.array_equal(got, ref), f"algo {algo}: pair lists differ"


def test_c3_shell_16m_build_and_uneven_knn():
    pts = bench.shell_points(16_000_000, 301)
    t = otg.Tree("points").create(pts, max_depth=10, max_elements=20)
    o = oracle().create(pts, KIND_POINTS, 10, None, 20, threads=THREADS)
    assert np.array_equal(t.location_keys(), o.location_keys())
    gn = t.nodes()
    assert len(gn["keys"]) > 3_000_000
    assert_nodes_equal_exact(gn, o.nodes(), "16M shell points")
    del gn
    q = bench.shell_points(1_000_000, 302)[:20_000]
    ks = np.random.default_rng(303).integers(1, 65, 1_000_000).astype(np.uint32)[:20_000]
    ref = _par(lambda x, k: o.knn(x, k), q, ks)
    for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
        assert_csr_equal(t.knn(q, ks, algo=algo), ref, f"uneven knn algo {algo}")
