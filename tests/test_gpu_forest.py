"""Forests: many independent trees built and queried in one call. Every tree of the forest must
equal the CPU oracle's tree of the same entities (node keys, node geometry, entity sets) and answer
every query exactly as that tree would, for point and box trees, FP64 and FP32, estimated and fixed
depths, given boxes and empty trees."""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import GPU_KIND, assert_csr_equal, assert_dist_close, assert_nodes_equal, node_dict
from _oracle_lib import KIND_BOXES, KIND_LOOSE_BOXES, KIND_POINTS, oracle

pytestmark = pytest.mark.gpu
RAY_REL = 1e-12


def _sizes(rng, trees, lo, hi):
    return np.clip(rng.lognormal(np.log((lo + hi) / 4), 1.0, trees), lo, hi).astype(np.int64)


def _forest_entities(kind, sizes, rng, dtype):
    parts = []
    for n in sizes:
        if kind == KIND_POINTS:
            parts.append(rng.random((n, 3)) * 100)
        else:
            c = rng.random((n, 3)) * 100
            e = rng.uniform(0.05, 1.0, (n, 3))
            parts.append(np.concatenate([c - e, c + e], 1))
    ent = np.concatenate(parts).astype(dtype) if parts else np.zeros((0, 3 if kind == KIND_POINTS else 6), dtype)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    return ent, off


def _split(res, qoff, t):
    """CSR of the queries of tree t."""
    off, ids = res[0], res[1]
    a, b = int(qoff[t]), int(qoff[t + 1])
    o = off[a : b + 1].astype(np.int64)
    sl = slice(int(o[0]), int(o[-1]))
    out = [o - o[0], ids[sl]]
    if len(res) > 2 and res[2] is not None:
        out.append(res[2][sl])
    return tuple(out)


def _queries(rng, trees, per, dtype):
    c = rng.random((trees * per, 3)) * 100
    e = rng.uniform(0.5, 5, (trees * per, 3))
    ranges = np.concatenate([c - e / 2, c + e / 2], 1).astype(dtype)
    pts = (rng.random((trees * per, 3)) * 100).astype(dtype)
    d = rng.normal(size=(trees * per, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([rng.random((trees * per, 3)) * 100, d], 1).astype(dtype)
    planes = np.zeros((trees, 6, 4))
    for t in range(trees):
        lo, hi = rng.random(3) * 40, 60 + rng.random(3) * 40
        for a in range(3):
            planes[t, 2 * a, 0], planes[t, 2 * a, 1 + a] = lo[a], 1.0
            planes[t, 2 * a + 1, 0], planes[t, 2 * a + 1, 1 + a] = -hi[a], -1.0
    qoff = np.arange(trees + 1, dtype=np.uint64) * per
    return ranges, pts, rays, planes.astype(dtype), qoff


@pytest.mark.parametrize(
    "kind,dtype,max_depth,given_box",
    [
        (KIND_LOOSE_BOXES, np.float32, 0, False),
        (KIND_LOOSE_BOXES, np.float64, 0, False),
        (KIND_POINTS, np.float64, 0, False),
        (KIND_POINTS, np.float32, 5, True),
        (KIND_LOOSE_BOXES, np.float64, 6, True),
        (KIND_BOXES, np.float32, 0, False),
        (KIND_BOXES, np.float64, 6, True),
    ],
)
def test_forest_matches_oracle_trees(kind, dtype, max_depth, given_box):
    rng = np.random.default_rng(91 + max_depth + (kind == KIND_POINTS))
    trees = 24
    sizes = _sizes(rng, trees, 200, 20000)
    sizes[3] = 0  # an empty tree
    ent, off = _forest_entities(kind, sizes, rng, dtype)
    boxes = None
    if given_box:
        boxes = np.tile(np.array([[-5.0, -5.0, -5.0, 105.0, 105.0, 105.0]]), (trees, 1)).astype(dtype)
    f = otg.Forest(GPU_KIND[kind], dtype).create(ent, off, max_depth=max_depth, boxes=boxes, max_elements=16)
    assert f.tree_count == trees
    ranges, pts, rays, planes, qoff = _queries(rng, trees, 40, dtype)
    res = {
        "range0": f.range_search(ranges, qoff, otg.RANGE_INSIDE),
        "range1": f.range_search(ranges, qoff, otg.RANGE_OVERLAP),
        "pick": f.pick_search(pts, qoff),
        "knn": f.knn(pts, qoff, 7),
        "frustum": f.frustum_culling(planes, np.arange(trees + 1, dtype=np.uint64)),
        "ray_all": f.ray_all(rays, qoff),
        "ray_first": f.ray_first(rays, qoff),
    }
    # node structure per tree
    nodes = f.nodes()
    nt = f.node_trees()
    for t in range(trees):
        a, b = int(off[t]), int(off[t + 1])
        o = oracle().create(ent[a:b], kind, max_depth, None if boxes is None else boxes[t], 16)
        if b > a:
            sel = np.nonzero(nt == t)[0]
            eoff = nodes["eoff"].astype(np.int64)
            sub_eoff = [0]
            sub_eids = []
            for i in sel:
                ids = nodes["eids"][eoff[i] : eoff[i + 1]].astype(np.int64) - a
                sub_eids.append(ids)
                sub_eoff.append(sub_eoff[-1] + len(ids))
            gpu = dict(keys=nodes["keys"][sel], min=nodes["min"][sel], size=nodes["size"][sel], eoff=np.array(sub_eoff, np.uint64),
                       eids=np.concatenate(sub_eids).astype(np.uint32) if sub_eids else np.zeros(0, np.uint32))
            assert_nodes_equal(gpu, o.nodes(), f"tree {t} nodes")
        s = slice(int(qoff[t]), int(qoff[t + 1]))
        assert_csr_equal(_split(res["range0"], qoff, t)[:2], o.range_search(ranges[s], 0), f"tree {t} range inside")
        assert_csr_equal(_split(res["range1"], qoff, t)[:2], o.range_search(ranges[s], 1), f"tree {t} range overlap")
        assert_csr_equal(_split(res["pick"], qoff, t)[:2], o.pick_search(pts[s]), f"tree {t} pick")
        assert_csr_equal(_split(res["knn"], qoff, t), o.knn(pts[s], 7), f"tree {t} knn")
        assert_csr_equal(_split(res["frustum"], np.arange(trees + 1), t)[:2], o.frustum(planes[t : t + 1]), f"tree {t} frustum")
        for name, first in (("ray_all", False), ("ray_first", True)):
            g = _split(res[name], qoff, t)
            r = o.ray(rays[s], first=first)
            assert_csr_equal(g[:2], r[:2], f"tree {t} {name}")
            assert_dist_close(g[2], r[2], RAY_REL, f"tree {t} {name}")


def test_forest_rejects_single_tree_calls_and_vice_versa():
    rng = np.random.default_rng(97)
    ent, off = _forest_entities(KIND_POINTS, np.array([100, 200]), rng, np.float64)
    f = otg.Forest("points").create(ent, off)
    with pytest.raises(otg.OtgError):
        otg.Tree.range_search(f, np.zeros((1, 6)))
    t = otg.Tree("points").create(ent)
    out = otg.C.c_void_p()
    qoff = np.array([0, 1], np.uint64)
    rng_box = np.zeros((1, 6))
    rc = otg.library().otg_forest_range_search(t.h, rng_box.ctypes.data_as(otg.C.c_void_p), qoff.ctypes.data_as(otg.C.c_void_p), 0, -1.0, 0,
                                               otg.C.byref(out), otg.MEM_HOST, None)
    assert rc == 1
