"""The oracle against the reference itself on the benchmark configurations at their full sizes,
on the inputs bench.py measures: the 1M uniform points with 2000 of their range boxes (both modes)
and 2000 kNN(k = 8) queries; the 4M clustered boxes with their whole self-collision pair list;
the 16M shell points with 2000 uneven-k kNN queries. Together with tests/test_gpu_fullsize.py
(the CUDA path against the oracle on the same inputs) this pins the GPU results at full size to
the reference. Runs only where the reference harness was built (oracle/_ref)."""
import numpy as np
import pytest

import bench
from _compare import assert_csr_equal, assert_nodes_equal, assert_nodes_equal_exact
from _oracle_lib import KIND_LOOSE_BOXES, KIND_POINTS, oracle, reference

pytestmark = pytest.mark.skipif(reference() is None, reason="reference harness not built here")


def test_nodes_equal_exact_helper():
    """The vectorised node comparison accepts a shuffled copy of the same tree and rejects a
    tree whose node holds one entity of another."""
    pts = np.random.default_rng(7).random((20_000, 3))
    ref = oracle().create(pts, KIND_POINTS, 6, None, 8).nodes()
    perm = np.random.default_rng(8).permutation(len(ref["keys"]))
    cnt = np.diff(ref["eoff"].astype(np.int64))[perm]
    eids = np.concatenate([ref["eids"][int(ref["eoff"][i]) : int(ref["eoff"][i + 1])][::-1] for i in perm])
    shuffled = dict(keys=ref["keys"][perm], min=ref["min"][perm], size=ref["size"][perm], eoff=np.concatenate([[0], np.cumsum(cnt)]).astype(np.uint64), eids=eids)
    assert_nodes_equal_exact(shuffled, ref, "shuffled")
    assert_nodes_equal(shuffled, ref, "shuffled")
    bad = dict(shuffled)
    bad["eids"] = eids.copy()
    i = int(np.flatnonzero(cnt > 0)[0])
    j = int(np.flatnonzero(cnt > 0)[-1])
    a, b = int(bad["eoff"][i]), int(bad["eoff"][j])
    bad["eids"][a], bad["eids"][b] = bad["eids"][b], bad["eids"][a]
    with pytest.raises(AssertionError):
        assert_nodes_equal_exact(bad, ref, "bad")


def test_c1_uniform_1m():
    pts, ranges, q = bench.c1_workload(2000, 2000)
    o = oracle().create(pts, KIND_POINTS, 10, None, 20, threads=8)
    r = reference().create(pts, KIND_POINTS, 10, None, 20)
    assert np.array_equal(o.location_keys(), r.location_keys())
    assert_nodes_equal_exact(o.nodes(), r.nodes(), "1M points")
    for mode in (0, 1):
        assert_csr_equal(o.range_search(ranges, mode), r.range_search(ranges, mode), f"range mode {mode}")
    assert_csr_equal(o.knn(q, 8), r.knn(q, 8), "knn k=8")


def test_c2_clustered_boxes_4m():
    boxes = bench.cluster_boxes(4_000_000, 201)
    o = oracle().create(boxes, KIND_LOOSE_BOXES, 12, None, 32, threads=8)
    r = reference().create(boxes, KIND_LOOSE_BOXES, 12, None, 32)
    assert np.array_equal(o.location_keys(), r.location_keys())
    assert_nodes_equal_exact(o.nodes(), r.nodes(), "4M boxes")
    assert np.array_equal(o.collide_self(), r.collide_self())


def test_c3_shell_16m():
    pts = bench.shell_points(16_000_000, 301)
    o = oracle().create(pts, KIND_POINTS, 10, None, 20, threads=8)
    r = reference().create(pts, KIND_POINTS, 10, None, 20)
    assert np.array_equal(o.location_keys(), r.location_keys())
    assert_nodes_equal_exact(o.nodes(), r.nodes(), "16M shell points")
    q = bench.shell_points(1_000_000, 302)[:2000]
    ks = np.random.default_rng(303).integers(1, 65, 1_000_000).astype(np.uint32)[:2000]
    assert_csr_equal(o.knn(q, ks), r.knn(q, ks), "uneven knn")
