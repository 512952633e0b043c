"""Bulk Insert into point trees: the oracle's restatement against the reference itself (Create, then
Insert of new points, once or twice): node keys, node geometry, entity sets, parent links (the
links Insert adds may skip levels) and range, pick and kNN results over the new structure. Runs
only where the reference harness was built (oracle/_ref)."""
import numpy as np
import pytest

from _compare import assert_csr_equal, assert_nodes_equal
from _insert_cases import insert_case
from _oracle_lib import KIND_POINTS, oracle, reference

pytestmark = pytest.mark.skipif(reference() is None, reason="reference harness not built here")


@pytest.mark.parametrize("seed", range(12))
def test_insert_points_matches_reference(seed):
    base, depth, box, max_elem, batches = insert_case(seed)
    o = oracle().create(base, KIND_POINTS, depth, box, max_elem)
    r = reference().create(base, KIND_POINTS, depth, box, max_elem)
    for b in batches:
        assert o.insert(b) and r.insert(b)
    on, rn = o.nodes(), r.nodes()
    assert np.array_equal(on["keys"], rn["keys"]), "node keys differ"
    assert_nodes_equal(on, rn, f"insert seed {seed}")
    assert np.array_equal(o.parents(), r.parents()), "parent links differ"
    rng = np.random.default_rng(seed + 100)
    c = rng.random((200, 3)) * 10
    e = rng.random((200, 3)) * 1.5
    ranges = np.concatenate([c - e, c + e], 1).astype(base.dtype)
    for mode in (0, 1):
        assert_csr_equal(o.range_search(ranges, mode), r.range_search(ranges, mode), f"range {mode}")
    q = (rng.random((200, 3)) * 10).astype(base.dtype)
    assert_csr_equal(o.knn(q, 9), r.knn(q, 9), "knn")
    allp = np.concatenate([base] + batches)
    assert_csr_equal(o.pick_search(allp[::37]), r.pick_search(allp[::37]), "pick")


def test_insert_refuses_points_outside_the_space():
    base = np.random.default_rng(1).random((500, 3)) * 10
    o = oracle().create(base, KIND_POINTS, 5, np.array([0.0, 0, 0, 10, 10, 10]), 8)
    before = o.node_count
    assert not o.insert(np.array([[1.0, 2.0, 3.0], [11.0, 5.0, 5.0]]))
    assert o.node_count == before
