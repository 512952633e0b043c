"""Seeded bulk-Insert cases shared by the oracle-vs-reference and GPU-vs-oracle Insert tests."""
import numpy as np


def new_points(rng, n, dtype):
    """Points inside [0, 10)^3: half uniform, half in a few tight clusters (deep new nodes)."""
    u = rng.random((n // 2, 3)) * 10
    c = rng.random((6, 3)) * 9.5 + 0.2
    cl = c[rng.integers(0, 6, n - n // 2)] + rng.normal(0, 0.01, (n - n // 2, 3))
    return np.clip(np.concatenate([u, cl]), 0.0, 9.999).astype(dtype)


def insert_case(seed):
    """(base points, max depth, box, max elements, [batches of new points]) in [0, 10)^3."""
    rng = np.random.default_rng(seed)
    dtype = np.float32 if seed % 3 == 2 else np.float64
    base = (rng.random((int(rng.integers(200, 6000)), 3)) * 10).astype(dtype)
    depth = int(rng.integers(3, 11))
    max_elem = int(rng.choice([1, 4, 8, 20, 64]))
    box = np.array([0.0, 0, 0, 10, 10, 10], dtype)
    batches = [new_points(rng, int(rng.integers(1, 5000)), dtype) for _ in range(1 + seed % 2)]
    return base, depth, box, max_elem, batches


def parent_keys(nodes):
    """Parent key of every node (0 for the root), nodes in ascending key order, from a breadth-first
    node export whose children are contiguous and allocated in node order (child_count)."""
    keys = nodes["keys"]
    cc = nodes["child_count"].astype(np.int64)
    parent = np.zeros(len(keys), np.uint64)
    parent[1:] = np.repeat(keys, cc)[: len(keys) - 1]
    assert int(cc.sum()) == len(keys) - 1, "child counts do not cover the nodes"
    order = np.argsort(keys, kind="stable")
    return parent[order]
