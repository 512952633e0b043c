"""Comparison helpers shared by the oracle and GPU parity tests."""
import glob
import os

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# the GPU tree kind of each oracle kind (0 points, 1 loose boxes, 2 regular boxes)
GPU_KIND = {0: "points", 1: "boxes", 2: "regular_boxes"}


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


def assert_nodes_equal_exact(gpu, ref, what):
    """assert_nodes_equal for trees of millions of nodes, vectorised: the GPU's reachable nodes
    (any order) must be exactly the reference's nodes (sorted by key, entity ids ascending per
    node), with the same min points, sizes and entity sets. Trees with orphan nodes (locations
    outside the grid) need assert_nodes_equal."""
    order = np.argsort(gpu["keys"], kind="stable")
    assert np.array_equal(gpu["keys"][order], ref["keys"]), f"{what}: node keys differ ({len(order)} vs {len(ref['keys'])} nodes)"
    assert np.array_equal(gpu["min"][order], ref["min"]), f"{what}: node min points differ"
    assert np.array_equal(gpu["size"][order], ref["size"]), f"{what}: node sizes differ"
    geoff = gpu["eoff"].astype(np.int64)
    cnt = np.diff(geoff)[order]
    assert np.array_equal(cnt, np.diff(ref["eoff"].astype(np.int64))), f"{what}: entity counts per node differ"
    # the GPU's entity ids node by node in key order, then sorted inside each node
    first = np.repeat(geoff[:-1][order] - np.concatenate([[0], np.cumsum(cnt)[:-1]]), cnt)
    ge = gpu["eids"][first + np.arange(int(cnt.sum()))]
    seg = np.repeat(np.arange(len(cnt)), cnt)
    ge = ge[np.lexsort((ge, seg))]
    assert np.array_equal(ge, ref["eids"]), f"{what}: entity sets of some nodes differ"


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


def static_storage_index(n, depth):
    """The node storage variant the reference's static Create picks: IsFit over
    GetMaxPossibleNodeCount (core/ot_static_linear_core.h:326-344, :370-376, :574-580)."""
    if n == 0:
        return 0
    node_num = lambda d: ((1 << (3 * d)) - 1) // 7
    full = min(depth, (n - 1).bit_length() // 3)
    m = min(node_num(full) + (depth - full) * n, node_num(depth))
    if m < 0xFF and n < 0xFF:
        return 0
    if m < 0xFFFF and n < 0xFFFF:
        return 1
    return 2


def static_archive_bytes(layout, is_box, dtype, n, depth, max_elem, space_min, space_size, entities=None):
    """The bytes of the reference's BinaryOutputArchive for a static tree with this layout
    (serialization.h:359-385, :433-438; serialization/binary_archive.h; serialization/stl/*.h):
    little-endian scalars, u32 size tags before every vector and std::array, std::monostate empty.
    entities: the Managed form's entity array, or None for the core alone."""
    T = np.dtype(dtype).newbyteorder("<")
    out = bytearray()
    u32 = lambda v: out.extend(np.uint32(v).astype("<u4").tobytes())

    def vec3_rows(rows, groups):
        # each row: `groups` std::arrays of 3 scalars, each after its size tag 3
        rows = np.asarray(rows, T).reshape(len(rows), groups, 3)
        rec = np.zeros((len(rows), groups), np.dtype([("tag", "<u4"), ("v", T, 3)]))
        rec["tag"] = 3
        rec["v"] = rows
        out.extend(rec.tobytes())

    u32(0)  # StaticLinearOrthoTreeCore version
    u32(0)  # OrthoTreeCoreBase version
    out.extend(np.uint64(max_elem).astype("<u8").tobytes())
    u32(depth)
    space_min = np.asarray(space_min, T)
    space_size = np.asarray(space_size, T)
    if is_box:
        vec3_rows(np.concatenate([space_min, space_size])[None], 2)  # m_nominalTreeBox {minPoint, size}
    else:
        u32(depth + 2)  # m_nodeSize (core/ot_base.h:121-134)
        lf = T.type(1)
        sizes = []
        for _ in range(depth + 2):
            sizes.append(space_size * lf)
            lf = T.type(lf * T.type(0.5))
        vec3_rows(sizes, 1)
    idx = static_storage_index(n, depth)
    u32(idx)
    w = ("<u1", "<u2", "<u4")[idx]
    cb = np.asarray(layout["child_begins"])
    u32(cb.size)
    out.extend(cb.astype(w).tobytes())
    seg = np.asarray(layout["segments"]).reshape(-1, 2)
    u32(seg.shape[0])
    out.extend(seg.astype(w).tobytes())
    dep = np.asarray(layout["depth"], np.uint8)
    u32(dep.size)
    out.extend(dep.tobytes())
    es = np.asarray(layout["entity_storage"])
    u32(es.size)
    out.extend(es.astype("<u4").tobytes())
    geo = np.asarray(layout["geometry"], T)
    u32(geo.shape[0])
    if geo.shape[0]:
        vec3_rows(geo, 2 if is_box else 1)
    if entities is not None:
        ent = np.asarray(entities, T)
        u32(ent.shape[0])
        if ent.shape[0]:
            vec3_rows(ent, 2 if is_box else 1)
    return bytes(out)


def space_of(ent, is_box, box=None):
    """The tree's space as Create finds it (given box, or the entities' bounding box) and its size
    Max - Min in the tree's scalar type (detail/si_grid.h:65-100)."""
    T = ent.dtype.type
    if box is not None:
        b = np.asarray(box, ent.dtype)
        mn, mx = b[:3], b[3:]
    elif ent.shape[0] == 0:
        # the bounding box of nothing is the inverted box (IGM::BoxInvertedInit): its size overflows
        big = np.finfo(ent.dtype).max
        mn, mx = np.full(3, big, ent.dtype), np.full(3, -big, ent.dtype)
        with np.errstate(over="ignore"):
            return mn, (mx - mn).astype(T)
    else:
        mn = ent[:, :3].min(axis=0)
        mx = (ent[:, 3:] if is_box else ent).max(axis=0)
    return mn, (mx - mn).astype(T)


def tree_is_equal_to_static(dyn, st, tol):
    """OrthoTreeQueryBase::IsEqualTo (core/ot_query.h:2149-2266) between a dynamic tree (nodes():
    keys with sentinel bit, min, size, entity offsets and ids) and a static linear layout: equal
    node counts, then from the roots: the same entity set per node, node boxes equal within `tol`,
    the same number of children, and children matched by the octant of their centre against the
    parent's centre, recursively."""
    keys = [int(k) for k in dyn["keys"]]
    idx = {k: i for i, k in enumerate(keys)}
    m = len(st["depth"])
    if len(keys) != m:
        return False
    cb = np.asarray(st["child_begins"], np.int64)
    seg = np.asarray(st["segments"], np.int64)
    es = np.asarray(st["entity_storage"])
    geo = np.asarray(st["geometry"], np.float64)
    if geo.shape[1] == 3:
        # MinPoint trees store no size: GetNodeSize(depth) is the tree size halved per depth
        # (core/ot_base.h:121-134; a power-of-two factor, so exact), the dynamic root's size
        root = dyn["size"][idx[1]] if 1 in idx else np.zeros(3)
        sizes = root[None, :] * (0.5 ** np.asarray(st["depth"], np.float64))[:, None]
        geo = np.concatenate([geo, sizes], 1)

    def dyn_children(k):
        return [idx[(k << 3) | c] for c in range(8) if ((k << 3) | c) in idx]

    def st_children(i):
        return list(range(cb[i], cb[i + 1])) if i + 1 < len(cb) else []

    def octant(cmin, csize, pmin, psize):
        cc, pc = cmin + csize * 0.5, pmin + psize * 0.5
        return sum(1 << d for d in range(3) if cc[d] > pc[d])

    def rec(di, si):
        a = np.sort(dyn["eids"][int(dyn["eoff"][di]) : int(dyn["eoff"][di + 1])])
        b = np.sort(es[seg[si, 0] : seg[si, 0] + seg[si, 1]])
        if not np.array_equal(a, b):
            return False
        dmin, dsize = dyn["min"][di], dyn["size"][di]
        smin, ssize = geo[si, :3], geo[si, 3:]
        if np.any(np.abs(dmin - smin) > tol) or np.any(np.abs((dmin + dsize) - (smin + ssize)) > tol):
            return False
        dc, sc = dyn_children(keys[di]), st_children(si)
        if len(dc) != len(sc):
            return False
        md = {octant(dyn["min"][c], dyn["size"][c], dmin, dsize): c for c in dc}
        ms = {octant(geo[c, :3], geo[c, 3:], smin, ssize): c for c in sc}
        if md.keys() != ms.keys():
            return False
        return all(rec(md[o], ms[o]) for o in md)

    return m == 0 or rec(idx[1], 0)


def moved_span(ent, rng, is_box):
    """A new span for the same tree: a fifth of the entities moved a little, a few moved far (out of
    their nodes and out of the space), and boxes resized."""
    out = ent.copy()
    n = len(ent)
    idx = rng.choice(n, n // 5, replace=False)
    shift = rng.normal(0, 0.02, (len(idx), 3)).astype(ent.dtype)
    far = rng.choice(n, max(1, n // 100), replace=False)
    fshift = rng.normal(0, 30, (len(far), 3)).astype(ent.dtype)
    if is_box:
        out[idx, :3] += shift
        out[idx, 3:] += shift * 1.5
        out[far, :3] += fshift
        out[far, 3:] += fshift
        out[:, 3:] = np.maximum(out[:, 3:], out[:, :3])
    else:
        out[idx] += shift
        out[far] += fshift
    return out
