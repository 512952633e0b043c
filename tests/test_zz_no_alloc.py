"""otg_knn_noalloc: the kNN entry point that allocates no memory, called through the C-ABI.

Its per-query slots must hold exactly what otg_knn returns for the same tree and queries (ids and
distances compared exactly, as every kNN parity test here does), on two calls in a row, for point
and box trees in both scalar types. This file is collected last so that it also runs after every
other test in the same process; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

import octree_gb300 as otg

pytestmark = pytest.mark.gpu

MAX_QUERIES = 1 << 20


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _noalloc(tree, q, k, cap, max_distance=-1.0, tol=-1.0):
    torch = pytest.importorskip("torch")
    nq = int(q.shape[0])
    counts = torch.full((nq,), 0xDEAD, dtype=torch.int32, device="cuda")
    ids = torch.full((max(nq * cap, 1),), -1, dtype=torch.int32, device="cuda")
    dist = torch.full((max(nq * cap, 1),), -1.0, dtype=torch.float64, device="cuda")
    rc = otg.library().otg_knn_noalloc(tree.h, _ptr(q), nq, k, max_distance, tol, cap, _ptr(counts), _ptr(ids), _ptr(dist), None)
    assert rc == 0, otg.library().otg_last_error()
    return counts.cpu().numpy().view(np.uint32), ids.cpu().numpy().view(np.uint32), dist.cpu().numpy()


def _expect_slots(ref, counts, ids, dist, cap, what):
    off, rid, rdist = ref
    lengths = np.diff(off.astype(np.int64))
    assert np.array_equal(counts.astype(np.int64), lengths), f"{what}: counts differ"
    for qi in range(len(lengths)):
        m = min(int(lengths[qi]), cap)
        a, b = int(off[qi]), int(off[qi]) + m
        assert np.array_equal(ids[qi * cap : qi * cap + m], rid[a:b]), f"{what}: ids of query {qi} differ"
        assert np.array_equal(dist[qi * cap : qi * cap + m], rdist[a:b]), f"{what}: distances of query {qi} differ"


@pytest.mark.parametrize(
    "kind,dtype,k,cap",
    [("points", np.float64, 8, 16), ("points", np.float32, 5, 8), ("boxes", np.float64, 6, 12), ("points", np.float64, 8, 4)],
)
def test_noalloc_knn_matches_knn(kind, dtype, k, cap):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(41)
    n = 200_000
    if kind == "points":
        ent = (rng.random((n, 3)) * 100).astype(dtype)
    else:
        lo = rng.random((n, 3)) * 100
        ent = np.concatenate([lo, lo + rng.random((n, 3)) * 0.5], 1).astype(dtype)
    tree = otg.Tree(kind, dtype).create(ent, max_depth=8, max_elements=20)
    tree.sync()
    q = (rng.random((3000, 3)) * 100).astype(dtype)
    q[:20] = np.round(q[:20])  # a few queries on lattice points
    ref = tree.knn(q, k)
    qd = torch.as_tensor(q, device="cuda")
    for call in range(2):
        counts, ids, dist = _noalloc(tree, qd, k, cap)
        _expect_slots(ref, counts, ids, dist, cap, f"{kind} {np.dtype(dtype).name} call {call}")


def test_noalloc_knn_ties_and_max_distance():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(42)
    pts = np.round(rng.random((20000, 3)) * 30)  # many exact ties: counts above k
    tree = otg.Tree("points").create(pts, max_depth=6, max_elements=8)
    tree.sync()
    q = np.round(rng.random((300, 3)) * 30) + 0.5
    qd = torch.as_tensor(q, device="cuda")
    for md in (-1.0, 0.75, 2.0):
        ref = tree.knn(q, 7, max_distance=md)
        for call in range(2):
            counts, ids, dist = _noalloc(tree, qd, 7, 32, max_distance=md)
            _expect_slots(ref, counts, ids, dist, 32, f"ties maxdist {md} call {call}")


def test_noalloc_knn_limits():
    torch = pytest.importorskip("torch")
    lib = otg.library()
    tree = otg.Tree("points").create(np.random.default_rng(43).random((1000, 3)))
    tree.sync()
    one = torch.zeros((1, 3), dtype=torch.float64, device="cuda")
    counts = torch.zeros((1,), dtype=torch.int32, device="cuda")
    # n_queries = 0 only performs the per-device set-up
    assert lib.otg_knn_noalloc(tree.h, None, 0, 4, -1.0, -1.0, 0, None, None, None, None) == 0
    # above the scratch capacity: rejected before any device work (the pointers are never read)
    rc = lib.otg_knn_noalloc(tree.h, _ptr(one), MAX_QUERIES + 1, 4, -1.0, -1.0, 0, _ptr(counts), None, None, None)
    assert rc == 1 and b"1048576" in lib.otg_last_error()
    rc = lib.otg_knn_noalloc(tree.h, _ptr(one), 1, 257, -1.0, -1.0, 0, _ptr(counts), None, None, None)
    assert rc == 6
    host = np.zeros((1, 3))
    rc = lib.otg_knn_noalloc(tree.h, host.ctypes.data_as(C.c_void_p), 1, 4, -1.0, -1.0, 0, _ptr(counts), None, None, None)
    assert rc == 1 and b"device memory" in lib.otg_last_error()
    # slot_capacity 0: counts only
    rc = lib.otg_knn_noalloc(tree.h, _ptr(one), 1, 4, -1.0, -1.0, 0, _ptr(counts), None, None, None)
    assert rc == 0 and int(counts[0]) == int(np.diff(tree.knn(one.cpu().numpy(), 4)[0].astype(np.int64))[0])


def test_noalloc_knn_empty_tree_and_k0():
    """An empty tree answers every query with count 0 (its own branch: no kernel runs), and k = 0
    gives empty lists on a non-empty tree; both over counts pre-filled with 0xDEAD, twice, and
    equal to otg_knn."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(44)
    q = rng.random((500, 3)) * 10
    qd = torch.as_tensor(q, device="cuda")
    empty = otg.Tree("points").create(np.zeros((0, 3)))
    empty.sync()
    full = otg.Tree("points").create(rng.random((50_000, 3)) * 10, max_depth=6, max_elements=16)
    full.sync()
    for tree, k, what in ((empty, 8, "empty tree"), (full, 0, "k = 0")):
        ref = tree.knn(q, k)
        assert int(ref[0][-1]) == 0
        for call in range(2):
            counts, ids, dist = _noalloc(tree, qd, k, 4)
            assert np.array_equal(counts, np.zeros(len(q), np.uint32)), f"{what} call {call}: counts not cleared"
            _expect_slots(ref, counts, ids, dist, 4, f"{what} call {call}")
