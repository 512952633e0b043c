"""Comparison helpers shared by the oracle and GPU parity tests."""
import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load_golden(name):
    with np.load(os.path.join(GOLDEN_DIR, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def assert_csr_equal(a, b, what):
    """a, b: (offsets, ids[, dist]) tuples; distances compared exactly unless rel_tol given."""
    assert np.array_equal(np.asarray(a[0], np.uint64), np.asarray(b[0], np.uint64)), f"{what}: offsets differ"
    assert np.array_equal(a[1], b[1]), f"{what}: ids differ ({len(a[1])} vs {len(b[1])})"
    if len(a) > 2 and len(b) > 2 and a[2] is not None and b[2] is not None:
        assert np.array_equal(a[2], b[2]), f"{what}: distances differ"


def assert_dist_close(a, b, rel, what):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape, f"{what}: distance count differs"
    err = np.abs(a - b) <= rel * np.maximum(np.abs(a), np.abs(b))
    assert err.all(), f"{what}: distances differ beyond {rel} relative"


def assert_nodes_equal(gpu, ref, what):
    """gpu: nodes reachable from the root (any order). ref: every node of the reference's node map,
    sorted by key. Nodes the reference holds but cannot reach from the root (its orphan nodes for
    locations outside the 3*D-bit grid) may only hold entities that no reachable node holds."""
    order = np.argsort(gpu["keys"], kind="stable")
    gk = gpu["keys"][order]
    rk = ref["keys"]
    pos = np.searchsorted(rk, gk)
    assert (pos < len(rk)).all() and np.array_equal(rk[np.minimum(pos, len(rk) - 1)], gk), f"{what}: node keys differ"
    assert np.array_equal(gpu["min"][order], ref["min"][pos]), f"{what}: node min points differ"
    assert np.array_equal(gpu["size"][order], ref["size"][pos]), f"{what}: node sizes differ"
    reached = set()
    for gi, ri in zip(order, pos):
        ge = np.sort(gpu["eids"][int(gpu["eoff"][gi]) : int(gpu["eoff"][gi + 1])])
        re = ref["eids"][int(ref["eoff"][ri]) : int(ref["eoff"][ri + 1])]
        assert np.array_equal(ge, re), f"{what}: entities of node {hex(int(gk[list(order).index(gi)]))} differ"
        reached.update(ge.tolist())
    extra = np.setdiff1d(np.arange(len(rk)), pos)
    for ri in extra:
        re = ref["eids"][int(ref["eoff"][ri]) : int(ref["eoff"][ri + 1])]
        assert not (set(re.tolist()) & reached), f"{what}: orphan node shares entities"


def node_dict(prefix, g):
    return {k: g[prefix + k] for k in ("keys", "min", "size", "eoff", "eids")}


def random_query_program(rng, nq, scale, dtype):
    """Combined-query inputs: per query 0-4 conditions (frustum of 1-6 planes with random crossing
    flags, range Inside / Overlap, plane intersection with the default or a 1% tolerance). Returns
    (conds, offsets, planes, crossing, boxes) in the layout of otg_query."""
    from _oracle_lib import COND_DTYPE, COND_FRUSTUM, COND_PLANE, COND_RANGE_INSIDE, COND_RANGE_OVERLAP

    conds, offsets, planes, crossing, boxes = [], [0], [], [], []

    def plane():
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        if rng.random() < 0.3:  # axis-aligned, on a node face
            n = np.eye(3)[rng.integers(0, 3)]
            return [np.round(rng.random() * 16) * scale / 16, *n]
        return [float(n @ (rng.random(3) * scale)), *n]

    for q in range(nq):
        k = 0 if q % 17 == 0 else int(rng.integers(1, 5))
        for _ in range(k):
            kind = int(rng.integers(0, 4))
            if kind == COND_FRUSTUM:
                m = int(rng.integers(1, 7))
                conds.append((COND_FRUSTUM, len(planes), m, 0, -1.0))
                for _ in range(m):
                    planes.append(plane())
                    crossing.append(int(rng.random() < 0.5))
            elif kind == COND_PLANE:
                conds.append((COND_PLANE, len(planes), 1, 0, -1.0 if rng.random() < 0.5 else 0.01 * scale))
                planes.append(plane())
                crossing.append(0)
            else:
                c = rng.random(3) * scale
                e = rng.uniform(0.05, 0.4, 3) * scale
                conds.append((COND_RANGE_INSIDE if kind == 1 else COND_RANGE_OVERLAP, len(boxes), 1, 0, -1.0))
                boxes.append([*(c - e / 2), *(c + e / 2)])
        offsets.append(len(conds))
    return (
        np.array(conds, COND_DTYPE),
        np.array(offsets, np.uint64),
        np.array(planes, dtype).reshape(-1, 4),
        np.array(crossing, np.uint8),
        np.array(boxes, dtype).reshape(-1, 6),
    )


STATIC_KEYS = ("child_begins", "segments", "depth", "entity_storage", "geometry")


def static_from_golden(g):
    """The reference's static layout stored in a fixture, or None where it is undefined."""
    if not int(g["static_defined"]):
        return None
    return {k: g["static_" + k] for k in STATIC_KEYS}


def assert_static_equal(a, b, what, exact_storage=False):
    """Static linear layouts (StaticLinearOrthoTreeCore's arrays) equal array for array: child
    segment begins as stored, entity segments, depth ids and node geometry bit for bit (geometry
    compared in double; float values widen exactly). Entity storage holds the same ids in every
    node's segment; exact_storage also asks for the same order inside segments (entities with
    equal locations are in id order on both sides unless one side is the reference, whose
    unstable sort leaves them unspecified)."""
    for k in ("child_begins", "segments", "depth"):
        assert a[k].shape == b[k].shape and np.array_equal(a[k], b[k]), f"{what}: static {k}"
    ga, gb = np.asarray(a["geometry"], np.float64), np.asarray(b["geometry"], np.float64)
    assert ga.shape == gb.shape and np.array_equal(ga, gb), f"{what}: static geometry"
    ea, eb = a["entity_storage"], b["entity_storage"]
    assert ea.shape == eb.shape, f"{what}: static entity storage size"
    if exact_storage:
        assert np.array_equal(ea, eb), f"{what}: static entity storage"
        return
    for bg, ln in a["segments"]:
        sa, sb = np.sort(ea[bg : bg + ln]), np.sort(eb[bg : bg + ln])
        assert np.array_equal(sa, sb), f"{what}: static entities of the segment at {bg}"
    assert np.array_equal(np.sort(ea), np.sort(eb)), f"{what}: static entity storage as a set"
