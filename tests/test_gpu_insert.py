"""Bulk Insert into GPU point trees against the oracle's restatement of the reference's Insert
(core/ot_dynamic_hash_core.h:1012-1333 with LinkOrphanNodes :826-863): the same Create, then the
same batches of new points, must give the same node keys, node geometry, entity sets, parent links
and query results (range in both modes, pick, kNN, frustum, rays), in the batched and the plain
kernels."""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import assert_csr_equal, assert_dist_close, assert_nodes_equal_exact
from _insert_cases import insert_case, new_points, parent_keys
from _oracle_lib import KIND_POINTS, oracle

pytestmark = pytest.mark.gpu

RAY_REL = 1e-12


def _pair(base, depth, box, max_elem):
    t = otg.Tree("points", base.dtype).create(base, max_depth=depth, box=box, max_elements=max_elem)
    o = oracle().create(base, KIND_POINTS, depth, box, max_elem)
    return t, o


def _check_structure(t, o, what):
    gn, on = t.nodes(), o.nodes()
    assert t.info().entity_count == o.n
    assert_nodes_equal_exact(gn, on, what)
    assert np.array_equal(parent_keys(gn), o.parents()), f"{what}: parent links differ"
    assert np.array_equal(t.location_keys(), o.location_keys()), f"{what}: location keys differ"


def _check_queries(t, o, rng, scale, nq, what):
    dtype = o.ent.dtype
    c = rng.random((nq, 3)) * scale
    e = rng.random((nq, 3)) * 0.15 * scale
    ranges = np.concatenate([c - e, c + e], 1).astype(dtype)
    for mode in (0, 1):
        ref = o.range_search(ranges, mode)
        for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
            assert_csr_equal(t.range_search(ranges, mode, algo=algo)[:2], ref, f"{what} range {mode} algo {algo}")
    q = (rng.random((nq, 3)) * scale).astype(dtype)
    ks = rng.integers(1, 40, nq).astype(np.uint32)
    ref = o.knn(q, ks)
    for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
        assert_csr_equal(t.knn(q, ks, algo=algo), ref, f"{what} knn algo {algo}")
    allp = o.ent
    picks = allp[:: max(1, len(allp) // nq)]
    assert_csr_equal(t.pick_search(picks)[:2], o.pick_search(picks), f"{what} pick")
    nrm = rng.normal(size=(8, 4, 3))
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    planes = np.concatenate([rng.random((8, 4, 1)) * scale * 0.5, nrm], 2).astype(dtype)
    assert_csr_equal(t.frustum_culling(planes)[:2], o.frustum(planes), f"{what} frustum")
    dirs = rng.normal(size=(nq, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rays = np.concatenate([rng.random((nq, 3)) * scale, dirs], 1).astype(dtype)
    tol = 5e-4 * scale
    for first in (False, True):
        g = t.ray_first(rays, tol=tol) if first else t.ray_all(rays, tol=tol)
        r = o.ray(rays, first=first, tol=tol)
        assert_csr_equal(g[:2], r[:2], f"{what} ray first={first}")
        assert_dist_close(g[2], r[2], RAY_REL, f"{what} ray first={first}")


@pytest.mark.parametrize("seed", range(12))
def test_insert_matches_oracle(seed):
    base, depth, box, max_elem, batches = insert_case(seed)
    t, o = _pair(base, depth, box, max_elem)
    for i, b in enumerate(batches):
        t.insert(b)
        assert o.insert(b)
        _check_structure(t, o, f"seed {seed} batch {i}")
    _check_queries(t, o, np.random.default_rng(seed + 500), 10.0, 300, f"seed {seed}")


@pytest.mark.parametrize(
    "dtype,depth,max_elem",
    [(np.float64, 10, 20), (np.float32, 10, 20), (np.float64, 19, 1), (np.float64, 6, 64), (np.float32, 16, 8)],
)
def test_insert_large_batches(dtype, depth, max_elem):
    """Hundreds of thousands of new points over a larger tree: several radix rounds, runs of
    identical locations longer than the 256-point walk limit, inserts into nodes at max depth."""
    rng = np.random.default_rng(depth * 7 + max_elem)
    base = (rng.random((300_000, 3)) * 100).astype(dtype)
    box = np.array([0.0, 0, 0, 100, 100, 100], dtype)
    t, o = _pair(base, depth, box, max_elem)
    dup = np.repeat((rng.random((3, 3)) * 100).astype(dtype), [300, 1000, 40], axis=0)
    add = np.concatenate([new_points(rng, 200_000, dtype) * dtype(10), dup, base[:5000]])
    add = add[rng.permutation(len(add))]
    t.insert(add)
    assert o.insert(add)
    _check_structure(t, o, "large batch")
    add2 = (rng.random((50_000, 3)) * 100).astype(dtype)
    t.insert(add2)
    assert o.insert(add2)
    _check_structure(t, o, "second batch")
    _check_queries(t, o, rng, 100.0, 2000, "large batch")


def test_insert_from_device_memory():
    torch = pytest.importorskip("torch")
    base, depth, box, max_elem, batches = insert_case(4)
    t1, o = _pair(base, depth, box, max_elem)
    t2 = otg.Tree("points", base.dtype).create(torch.from_numpy(base).cuda(), max_depth=depth, box=box, max_elements=max_elem)
    for b in batches:
        t1.insert(b)
        t2.insert(torch.from_numpy(b).cuda())
        assert o.insert(b)
    _check_structure(t2, o, "device insert")
    a, b = t1.nodes(), t2.nodes()
    assert np.array_equal(a["keys"], b["keys"]) and np.array_equal(a["eids"], b["eids"])


def test_insert_refuses_points_outside_and_changes_nothing():
    base, depth, box, max_elem, batches = insert_case(0)
    t, o = _pair(base, depth, box, max_elem)
    before = t.nodes()
    bad = np.concatenate([batches[0][:10], np.array([[11.0, 5.0, 5.0]], base.dtype)])
    with pytest.raises(otg.OtgError):
        t.insert(bad)
    after = t.nodes()
    assert t.info().entity_count == len(base)
    for k in ("keys", "eoff", "eids", "child_count"):
        assert np.array_equal(before[k], after[k])
    # the tree still takes a valid batch afterwards
    t.insert(batches[0])
    assert o.insert(batches[0])
    _check_structure(t, o, "after a refused batch")


def test_insert_edge_cases():
    base, depth, box, max_elem, _ = insert_case(3)
    t, o = _pair(base, depth, box, max_elem)
    t.insert(np.zeros((0, 3), base.dtype))
    assert t.info().entity_count == len(base)
    one = np.array([[5.0, 5.0, 5.0]], base.dtype)
    t.insert(one)
    assert o.insert(one)
    _check_structure(t, o, "one point")
    corner = np.array([[0.0, 0.0, 0.0], [9.999, 9.999, 9.999], [10.0, 10.0, 10.0]], base.dtype)
    t.insert(corner)
    assert o.insert(corner)
    _check_structure(t, o, "corners")
    # the static layout is a Create's: refused after Insert
    with pytest.raises(otg.OtgError):
        t.export_static()
    # an empty tree has no space to insert into
    e = otg.Tree("points").create(np.zeros((0, 3)), max_depth=4, box=np.array([0.0, 0, 0, 1, 1, 1]), max_elements=4)
    with pytest.raises(otg.OtgError):
        e.insert(np.array([[0.5, 0.5, 0.5]]))
    # box trees have no Insert here
    b = otg.Tree("boxes").create(np.array([[0.0, 0, 0, 1, 1, 1], [2.0, 2, 2, 3, 3, 3]]), max_depth=3, max_elements=1)
    with pytest.raises(otg.OtgError):
        b.insert(np.array([[0.5, 0.5, 0.5, 0.6, 0.6, 0.6]]))


def test_core_form_after_insert():
    """The Core form's moved span also works after an Insert (set_entities takes the new count)."""
    base, depth, box, max_elem, batches = insert_case(5)
    t, o = _pair(base, depth, box, max_elem)
    for b in batches:
        t.insert(b)
        assert o.insert(b)
    rng = np.random.default_rng(9)
    moved = np.clip(o.ent + rng.normal(0, 0.002, o.ent.shape), 0, 9.999).astype(o.ent.dtype)
    t.set_entities(moved)
    o.set_entities(moved)
    c = rng.random((200, 3)) * 10
    e = rng.random((200, 3)) * 1.5
    ranges = np.concatenate([c - e, c + e], 1).astype(moved.dtype)
    for mode in (0, 1):
        assert_csr_equal(t.range_search(ranges, mode)[:2], o.range_search(ranges, mode), f"core range {mode}")
