"""Properties of the tree after a bulk Insert that the device Insert relies on, checked on the
oracle's restatement of the reference's Insert (core/ot_dynamic_hash_core.h:1012-1333 with
LinkOrphanNodes :826-863), in depth-first (pre-order) node order:

* the node set is closed under lowest common ancestors of depth-first neighbours;
* the parent of every node but the root is the lowest common ancestor of the node and its
  depth-first predecessor;
* every child sits in a distinct child slot of its parent."""
import numpy as np
import pytest

from _insert_cases import insert_case
from _oracle_lib import KIND_POINTS, oracle


def key_depth(k):
    return (k.bit_length() - 1) // 3


def dfs_key(k, D):
    """location left-aligned to the max depth, then depth (pre-order of the octree)"""
    d = key_depth(k)
    return (((k ^ (1 << (3 * d))) << (3 * (D - d))) << 5) | d


def lca(a, b):  # si_morton.h:307-325
    if a == b:
        return a
    da, db = key_depth(a), key_depth(b)
    if da > db:
        a >>= 3 * (da - db)
    elif db > da:
        b >>= 3 * (db - da)
    return a >> (3 * (((a ^ b).bit_length() + 2) // 3))


@pytest.mark.parametrize("seed", range(12))
def test_inserted_tree_is_an_lca_closed_trie(seed):
    base, depth, box, max_elem, batches = insert_case(seed)
    o = oracle().create(base, KIND_POINTS, depth, box, max_elem)
    for b in batches:
        assert o.insert(b)
    D = o.max_depth
    keys = [int(k) for k in o.nodes()["keys"]]
    parents = dict(zip(keys, (int(p) for p in o.parents())))
    order = sorted(keys, key=lambda k: dfs_key(k, D))
    present = set(keys)
    assert order[0] == 1 and parents[1] == 0
    slots = set()
    for prev, k in zip(order, order[1:]):
        p = lca(prev, k)
        assert p in present, f"seed {seed}: lowest common ancestor {hex(p)} missing"
        assert parents[k] == p, f"seed {seed}: parent of {hex(k)} is {hex(parents[k])}, not {hex(p)}"
        slot = (k >> (3 * (key_depth(k) - key_depth(p) - 1))) & 7  # si_morton.h:651-658
        assert (p, slot) not in slots
        slots.add((p, slot))
