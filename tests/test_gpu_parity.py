"""Parity of the CUDA path with the reference (golden fixtures) and with the CPU oracle on seeded
inputs. Ids must match exactly; ray and kNN distances are compared bit-exact except where stated
(ray hit distances: 1e-12 relative, as the parity bar for FP64 ray distances states)."""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import (
    GPU_KIND,
    assert_csr_equal,
    assert_dist_close,
    assert_nodes_equal,
    assert_nodes_equal_exact,
    golden_cases,
    load_golden,
    moved_span,
    node_dict,
)
from _oracle_lib import KIND_BOXES, KIND_LOOSE_BOXES, KIND_POINTS, oracle

pytestmark = pytest.mark.gpu

RAY_REL = 1e-12


def _gpu_tree(ent, kind, max_depth, box, max_elem):
    t = otg.Tree(GPU_KIND[kind], ent.dtype)
    return t.create(ent, max_depth=max_depth, box=box, max_elements=max_elem)


def _check_queries(t, o, q, kind, ray_tol, what):
    for mode in (0, 1):
        assert_csr_equal(t.range_search(q["ranges"], mode)[:2], o.range_search(q["ranges"], mode), f"{what} range{mode}")
    assert_csr_equal(t.pick_search(q["qpts"])[:2], o.pick_search(q["qpts"]), f"{what} pick")
    g = t.knn(q["qpts"], q["k"])
    r = o.knn(q["qpts"], q["k"])
    assert_csr_equal(g, r, f"{what} knn")
    assert_csr_equal(t.frustum_culling(q["planes"])[:2], o.frustum(q["planes"]), f"{what} frustum")
    for first in (False, True):
        g = t.ray_first(q["rays"], tol=ray_tol) if first else t.ray_all(q["rays"], tol=ray_tol)
        r = o.ray(q["rays"], first=first, tol=ray_tol)
        assert_csr_equal(g[:2], r[:2], f"{what} ray first={first}")
        assert_dist_close(g[2], r[2], RAY_REL, f"{what} ray first={first}")


@pytest.mark.parametrize("name", golden_cases())
def test_gpu_matches_reference_fixture(name):
    g = load_golden(name)
    kind = int(g["kind"])
    t = _gpu_tree(g["entities"], kind, int(g["max_depth"]), g.get("box"), int(g["max_elem"]))
    assert t.max_depth == int(g["depth"])
    assert np.array_equal(t.location_keys(), g["loc"])
    assert_nodes_equal(t.nodes(), node_dict("node_", g), name)
    for mode in (0, 1):
        assert_csr_equal(t.range_search(g["ranges"], mode)[:2], (g[f"range{mode}_off"], g[f"range{mode}_ids"]), f"range{mode}")
    assert_csr_equal(t.pick_search(g["qpts"])[:2], (g["pick_off"], g["pick_ids"]), "pick")
    assert_csr_equal(t.knn(g["qpts"], g["k"]), (g["knn_off"], g["knn_ids"], g["knn_dist"]), "knn")
    assert_csr_equal(t.frustum_culling(g["planes"])[:2], (g["frustum_off"], g["frustum_ids"]), "frustum")
    for first in (0, 1):
        fn = t.ray_first if first else t.ray_all
        res = fn(g["rays"], tol=float(g["ray_tol"]))
        assert_csr_equal(res[:2], (g[f"ray{first}_off"], g[f"ray{first}_ids"]), f"ray{first}")
        assert_dist_close(res[2], g[f"ray{first}_dist"], RAY_REL, f"ray{first}")
    if kind != KIND_POINTS:
        assert np.array_equal(t.collision_self(), g["collide"])
        t2 = _gpu_tree(g["other"], kind, int(g["max_depth"]), None, int(g["max_elem"]))
        assert np.array_equal(t.collision_pair(t2), g["collide_pair"])


def _queries(rng, dtype, scale, nq=400):
    c = rng.random((nq, 3)) * scale * 1.1 - 0.05 * scale
    e = rng.random((nq, 3)) * 0.06 * scale
    ranges = np.concatenate([c - e, c + e], 1).astype(dtype)
    pts = (rng.random((nq, 3)) * scale).astype(dtype)
    k = rng.integers(1, 65, nq).astype(np.uint32)
    nrm = rng.normal(size=(16, 6, 3))
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    planes = np.concatenate([rng.random((16, 6, 1)) * scale * 0.6 - 0.3 * scale, nrm], 2).astype(dtype)
    dirs = rng.normal(size=(nq, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rays = np.concatenate([rng.random((nq, 3)) * scale, dirs], 1).astype(dtype)
    return dict(ranges=ranges, qpts=pts, k=k, planes=planes, rays=rays)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("max_depth,max_elem", [(10, 20), (0, 16), (5, 4), (19, 32)])
def test_points_random(dtype, max_depth, max_elem):
    rng = np.random.default_rng(max_depth * 100 + max_elem)
    pts = (rng.random((200_000, 3)) * 100).astype(dtype)
    t = _gpu_tree(pts, KIND_POINTS, max_depth, None, max_elem)
    o = oracle().create(pts, KIND_POINTS, max_depth, None, max_elem)
    assert t.max_depth == o.max_depth
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal(t.nodes(), o.nodes(), "points")
    _check_queries(t, o, _queries(rng, dtype, 100), KIND_POINTS, 0.05, "points")


def _emission_case(name):
    rng = np.random.default_rng(77)
    if name == "all_outside":
        return rng.random((5000, 3)) * 50 + 100, np.array([0.0, 0, 0, 50, 50, 50]), 10, 8
    if name == "partly_outside":
        return rng.random((40_000, 3)) * 100, np.array([20.0, 20, 20, 70, 70, 70]), 9, 12
    if name in ("n_eq_max", "n_above_max"):
        n = 64 if name == "n_eq_max" else 65
        return rng.random((n, 3)), None, 6, 64
    if name in ("dup_run_d10", "dup_run_d19"):
        # identical points spanning several tiles of sorted keys: a chain down to the deepest depth
        pts = np.concatenate([np.repeat([[0.3, 0.6, 0.2]], 5000, 0), rng.random((3000, 3)), np.repeat([[0.9, 0.1, 0.5]], 2100, 0)])
        return pts, None, 10 if name == "dup_run_d10" else 19, 8
    if name in ("max_elem_1024", "max_elem_1025"):
        return rng.random((60_000, 3)) * 10, None, 8, 1024 if name == "max_elem_1024" else 1025
    if name == "clusters_big":
        # tight clusters: depth-B cells of tens of thousands of points, split cell by cell
        c = rng.random((4, 3))
        pts = np.concatenate([c[rng.integers(0, 4, 100_000)] + rng.normal(0, 0.002, (100_000, 3)), rng.random((100_000, 3))])
        return pts, None, 10, 20
    if name == "dup_big":
        # one depth-D cell holding more points than a block handles in shared memory
        return np.concatenate([np.repeat([[0.41, 0.52, 0.63]], 20_000, 0), rng.random((5000, 3))]), None, 10, 8
    if name == "pairs_max_elem_1":
        # near-identical pairs with maxElementNo 1: node chains down to where each pair separates
        # (more nodes than positions in a work item)
        p0 = rng.random((30_000, 3))
        return np.concatenate([p0, p0 + rng.normal(0, 2e-4, p0.shape)]), None, 10, 1
    if name == "shell":
        n = 300_000
        u = rng.random((n * 7 // 10, 3))
        d = rng.normal(size=(n - len(u), 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        return np.concatenate([u, 0.5 + d * rng.normal(0.4, 0.005, (len(d), 1))]), None, 12, 20
    raise KeyError(name)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize(
    "name",
    ["all_outside", "partly_outside", "n_eq_max", "n_above_max", "dup_run_d10", "dup_run_d19", "max_elem_1024", "max_elem_1025", "shell",
     "clusters_big", "dup_big", "pairs_max_elem_1"],
)
def test_point_emission_layouts(dtype, name):
    """Point-tree node emission on layouts that stress it: outside points held by the root, a root
    at the split threshold, runs of identical points crossing sorted-key tiles down to the deepest
    depth, the largest and smallest maxElementNo of each emission method, a dense shell, buckets
    above one block's shared-memory capacity (tight clusters, one cell of identical points), and
    more nodes than positions (near-identical pairs, maxElementNo 1)."""
    pts, box, max_depth, max_elem = _emission_case(name)
    pts = pts.astype(dtype)
    box = None if box is None else box.astype(dtype)
    t = _gpu_tree(pts, KIND_POINTS, max_depth, box, max_elem)
    o = oracle().create(pts, KIND_POINTS, max_depth, box, max_elem)
    assert t.max_depth == o.max_depth
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal(t.nodes(), o.nodes(), name)
    rng = np.random.default_rng(5)
    lo, hi = pts.min(0), pts.max(0)
    c = lo + rng.random((200, 3)) * (hi - lo)
    e = rng.random((200, 3)) * (hi - lo) * 0.05
    ranges = np.concatenate([c - e, c + e], 1).astype(dtype)
    for mode in (0, 1):
        assert_csr_equal(t.range_search(ranges, mode)[:2], o.range_search(ranges, mode), f"{name} range{mode}")
    q = c.astype(dtype)
    assert_csr_equal(t.knn(q, 9), o.knn(q, 9), f"{name} knn")


@pytest.mark.parametrize("max_depth", [8, 9, 10])
@pytest.mark.parametrize("n", [1, 2, 100, 4095, 4096, 4097, 12289, 70_001])
def test_point_sort_tile_boundaries(max_depth, n):
    """Radix-sort tiles of 4096 keys: one key, one tile, a partial last tile, sizes either side of
    a tile boundary, and a run of identical keys across tiles, in the data's bounding box and in a
    given box, against the oracle."""
    rng = np.random.default_rng(n * 16 + max_depth)
    pts = rng.random((n, 3))
    if n > 10:
        pts[: n // 10] = pts[n // 2]  # a run of identical keys across tiles
    for box in (None, np.array([0.0, 0, 0, 1, 1, 1])):
        t = _gpu_tree(pts, KIND_POINTS, max_depth, box, 4)
        o = oracle().create(pts, KIND_POINTS, max_depth, box, 4)
        assert np.array_equal(t.location_keys(), o.location_keys())
        assert_nodes_equal(t.nodes(), o.nodes(), f"n={n} depth {max_depth} box {box is not None}")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("max_depth", [10, 12])
@pytest.mark.parametrize("offset", [0.0, 819.0, 1e6])
def test_point_cells_near_boundaries(dtype, max_depth, offset):
    """Point cells from the FP32 estimate where it clears its rounding margin, from the threshold
    tables elsewhere: coordinates on cell boundaries, a few ulps either side, at distances around
    the margin, and full-mantissa values within two margins of a boundary, in a space whose
    boundaries are not short binary fractions. The margin grows with the coordinates' magnitude: at
    an offset of 1e6 it leaves about half of the coordinates to the tables at depth 10 and switches
    the estimate off at depth 12. In a given box and in the points' own box, against the oracle
    (tests/test_cell_estimate_margin.py checks the same estimate on the CPU, and that these inputs
    need the margin)."""
    rng = np.random.default_rng(int(offset) + max_depth)
    cells = 1 << max_depth
    size, low = 1000.123456789, offset + 0.3712345
    width = size / cells
    j = rng.integers(0, cells + 1, (60_000, 3)).astype(np.float64)
    x = low + j * width
    k = rng.integers(-4, 5, x.shape)
    for step in range(4):  # up to four ulps either side
        x = np.where(k > step, np.nextafter(x, np.inf), np.where(k < -step, np.nextafter(x, -np.inf), x))
    margin = (size + offset) * (cells / size) * 2.0**-22 + cells * 2.0**-22
    near = low + (j + rng.choice([-2.0, -1.0, -0.5, 0.5, 1.0, 2.0], j.shape) * margin) * width
    band = low + (j + (rng.random(j.shape) * 2.0 - 1.0) * 2.0 * margin) * width
    pts = np.concatenate([x, near, band, low + rng.random((60_000, 3)) * size])
    pts = np.clip(pts, low, low + size).astype(dtype)
    for box in (None, np.array([low] * 3 + [low + size] * 3, dtype)):
        t = _gpu_tree(pts, KIND_POINTS, max_depth, box, 16)
        o = oracle().create(pts, KIND_POINTS, max_depth, box, 16)
        assert np.array_equal(t.location_keys(), o.location_keys()), f"box {box is not None}"
        assert_nodes_equal(t.nodes(), o.nodes(), f"offset {offset} box {box is not None}")


@pytest.mark.parametrize("kind", [KIND_LOOSE_BOXES, KIND_BOXES])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("max_depth,max_elem", [(8, 32), (0, 16), (4, 2)])
def test_boxes_random(dtype, max_depth, max_elem, kind):
    """Loose (OctreeBox) and regular (OctreeBoxs<false>) box trees against the oracle."""
    rng = np.random.default_rng(7 + max_depth + max_elem)
    n = 60_000
    cen = np.where(rng.random((n, 1)) < 0.5, rng.random((n, 3)) * 1000, rng.normal(500, 10, (n, 3)))
    half = rng.lognormal(np.log(0.5), 0.6, (n, 3))
    boxes = np.concatenate([cen - half, cen + half], 1).astype(dtype)
    t = _gpu_tree(boxes, kind, max_depth, None, max_elem)
    o = oracle().create(boxes, kind, max_depth, None, max_elem)
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal(t.nodes(), o.nodes(), "boxes")
    _check_queries(t, o, _queries(rng, dtype, 1000), kind, 0.0, "boxes")
    assert np.array_equal(t.collision_self(), o.collide_self())
    other = boxes.copy()
    other += dtype(0.4)
    t2 = _gpu_tree(other, kind, max_depth, None, max_elem)
    o2 = oracle().create(other, kind, max_depth, None, max_elem)
    assert np.array_equal(t.collision_pair(t2), o.collide_pair(o2))


def _gap_boxes(dtype, seed):
    """Boxes with coordinates in [140, 200], where the tolerance lies between half an ulp and an ulp,
    half of them starting one ulp after other boxes end in x: exercises the rounding gap of
    GetBoxRelation against the reference's sweep-and-prune."""
    rng = np.random.default_rng(seed)
    n = 3000
    cen = rng.random((n, 3)) * 60 + 140
    half = np.round(rng.random((n, 3)) * 4 + 0.5, 1)
    ent = np.concatenate([cen - half, cen + half], 1).astype(dtype)
    ent[n // 2 :, 0] = ent[: n - n // 2, 3]
    ent[n // 2 :, 3] = ent[n // 2 :, 0] + dtype(2.0)
    ent[n // 2 :, 0] = np.nextafter(ent[n // 2 :, 0], dtype(1e9))
    ent[n // 2 :, 3] = np.maximum(ent[n // 2 :, 3], ent[n // 2 :, 0])
    return ent


@pytest.mark.parametrize("kind", [KIND_LOOSE_BOXES, KIND_BOXES])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("max_depth,max_elem", [(3, 4), (5, 8), (2, 2)])
def test_collision_rounding_gap(dtype, max_depth, max_elem, kind):
    ent = _gap_boxes(dtype, 500 + max_depth)
    t = _gpu_tree(ent, kind, max_depth, None, max_elem)
    o = oracle().create(ent, kind, max_depth, None, max_elem)
    assert np.array_equal(t.collision_self(), o.collide_self())
    other = ent.copy()
    other[:, [0, 3]] = other[:, [0, 3]] + (other[:, 3:4] - other[:, 0:1])
    t2 = _gpu_tree(other, kind, max_depth, None, max_elem)
    o2 = oracle().create(other, kind, max_depth, None, max_elem)
    assert np.array_equal(t.collision_pair(t2), o.collide_pair(o2))
    assert np.array_equal(t2.collision_pair(t), o2.collide_pair(o))


EDGE_CASES = {
    "single": (np.array([[1.0, 2.0, 3.0]]), KIND_POINTS, None),
    "two_equal": (np.array([[1.0, 2.0, 3.0], [1.0, 2.0, 3.0]]), KIND_POINTS, None),
    "duplicates": (np.repeat(np.random.default_rng(3).random((40, 3)) * 10, 25, axis=0), KIND_POINTS, None),
    "flat": (np.c_[np.random.default_rng(4).random((3000, 2)) * 10, np.zeros(3000)], KIND_POINTS, None),
    "outside_box": (np.random.default_rng(5).random((3000, 3)) * 100, KIND_POINTS, np.array([10.0, 10, 10, 60, 60, 60])),
    "negative": (np.random.default_rng(6).random((3000, 3)) * 200 - 100, KIND_POINTS, None),
    "tiny_extent": (np.random.default_rng(8).random((3000, 3)) * 1e-9 + 1e5, KIND_POINTS, None),
}


def _edge_boxes():
    rng = np.random.default_rng(9)
    cen = rng.random((2000, 3)) * 50
    hh = rng.random((2000, 3)) * 4
    b = np.concatenate([cen - hh, cen + hh], 1)
    span = b.copy()
    span[0] = [b[:, 0].min(), b[:, 1].min(), b[:, 2].min(), b[:, 3].max(), b[:, 4].max(), b[:, 5].max()]
    corner = b.copy()
    corner[1] = [50, 50, 50, 50, 50, 50]
    corner[2] = [0, 0, 0, 0, 0, 0]
    # regular trees: boxes whose max corner falls exactly on a cell boundary (the reference steps the
    # max cell back there, si_grid.h:207-211), at the space's max face, and spanning several cells
    grid = np.floor(rng.random((1500, 3)) * 64) * (50 / 64)
    steps = rng.integers(0, 4, (1500, 3)) * (50 / 64)
    on_grid = np.concatenate([grid, np.minimum(grid + steps, 50.0)], 1)
    cases = {
        "boxes_degenerate": (np.concatenate([cen, cen], 1), KIND_LOOSE_BOXES, None),
        "box_spans_space": (span, KIND_LOOSE_BOXES, None),
        "boxes_on_max_corner": (corner, KIND_LOOSE_BOXES, np.array([0.0, 0, 0, 50, 50, 50])),
        "boxes_outside_box": (b, KIND_LOOSE_BOXES, np.array([10.0, 10, 10, 40, 40, 40])),
        "regular_boxes_on_cell_boundaries": (on_grid, KIND_BOXES, np.array([0.0, 0, 0, 50, 50, 50])),
    }
    # (a regular tree refuses a box with its min corner on the max face of the space, where the
    # reference asserts: test_regular_boxes_on_max_face_are_refused)
    for name in ("box_spans_space", "boxes_outside_box"):
        ent, _, box = cases[name]
        cases["regular_" + name] = (ent, KIND_BOXES, box)
    return cases


@pytest.mark.parametrize("name", list(EDGE_CASES) + list(_edge_boxes()))
@pytest.mark.parametrize("max_depth,max_elem", [(0, 1), (3, 4), (10, 16)])
def test_edge_cases(name, max_depth, max_elem):
    ent, kind, box = {**EDGE_CASES, **_edge_boxes()}[name]
    t = _gpu_tree(ent, kind, max_depth, box, max_elem)
    o = oracle().create(ent, kind, max_depth, box, max_elem)
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal(t.nodes(), o.nodes(), name)
    rng = np.random.default_rng(11)
    lo = ent[:, :3].min(0)
    hi = ent[:, 3:].max(0) if kind != KIND_POINTS else ent.max(0)
    span = np.maximum(hi - lo, 1e-12)
    c = lo + rng.random((64, 3)) * span
    e = rng.random((64, 3)) * span * 0.2
    ranges = np.concatenate([c - e, c + e], 1)
    ranges[0] = np.concatenate([lo - 1, hi + 1])  # whole-tree range: root shortcut
    ranges[1] = np.concatenate([c[1], c[1]])  # zero volume
    for mode in (0, 1):
        assert_csr_equal(t.range_search(ranges, mode)[:2], o.range_search(ranges, mode), f"{name} range{mode}")
    q = np.concatenate([ent[:16, :3], c[:16]])
    assert_csr_equal(t.knn(q, 5), o.knn(q, 5), f"{name} knn")
    assert_csr_equal(t.pick_search(q)[:2], o.pick_search(q), f"{name} pick")
    if kind != KIND_POINTS:
        assert np.array_equal(t.collision_self(), o.collide_self())


def test_regular_boxes_on_max_face_are_refused():
    """A regular (non-loose) box tree refuses a box whose min corner rasterises to cell 2^D (on the
    max face of the space within the tolerance): the reference asserts there (detail/si_grid.h:213)
    and its location's depth would wrap. Loose trees take such boxes (they hold them in no node)."""
    rng = np.random.default_rng(9)
    cen = rng.random((2000, 3)) * 50
    degenerate = np.concatenate([cen, cen], 1)  # its bounding box puts one of them on the max face
    corner = np.concatenate([cen - 1, cen + 1], 1)
    corner[1] = [50, 50, 50, 50, 50, 50]
    for ent, box in ((degenerate, None), (corner, np.array([0.0, 0, 0, 50, 50, 50]))):
        with pytest.raises(otg.OtgError):
            _gpu_tree(ent, KIND_BOXES, 5, box, 8)
        _gpu_tree(ent, KIND_LOOSE_BOXES, 5, box, 8)  # the loose tree takes them
    # the refusal comes from the same arithmetic the oracle restates: its location has a wrapped depth
    keys = oracle().create(degenerate, KIND_BOXES, 5, None, 8).location_keys()
    assert ((keys & 31) > 5).any()


def test_empty_tree():
    t = otg.Tree("points").create(np.zeros((0, 3)))
    off, ids, _ = t.range_search(np.array([[0.0, 0, 0, 1, 1, 1]]))
    assert len(ids) == 0 and off.tolist() == [0, 0]
    off, ids, d = t.knn(np.array([[0.0, 0, 0]]), 3)
    assert len(ids) == 0
    tb = otg.Tree("boxes").create(np.zeros((0, 6)))
    assert tb.collision_self().shape == (0, 2)


def test_knn_max_distance_and_ties():
    rng = np.random.default_rng(12)
    pts = np.round(rng.random((20000, 3)) * 30)  # many exact ties
    t = _gpu_tree(pts, KIND_POINTS, 6, None, 8)
    o = oracle().create(pts, KIND_POINTS, 6, None, 8)
    q = np.round(rng.random((200, 3)) * 30) + 0.5
    for md in (-1.0, 0.75, 2.0):
        assert_csr_equal(t.knn(q, 7, max_distance=md), o.knn(q, 7, max_dist=md), f"knn maxdist {md}")


def test_device_inputs_match_host_inputs():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(13)
    pts = rng.random((100_000, 3)) * 100
    th = otg.Tree("points").create(pts, max_depth=9, max_elements=20)
    td = otg.Tree("points").create(torch.as_tensor(pts, device="cuda"), max_depth=9, max_elements=20)
    td.sync()
    assert np.array_equal(th.location_keys(), td.location_keys())
    c = rng.random((100, 3)) * 100
    ranges = np.concatenate([c - 2, c + 2], 1)
    a = th.range_search(ranges)
    b = td.range_search(torch.as_tensor(ranges, device="cuda"))
    assert_csr_equal(a[:2], b[:2], "device input")


def test_device_inputs_at_unaligned_offsets():
    """Entities handed over as device views that start 8 bytes past a 16-byte boundary (a slice of a
    larger tensor) take the scalar loads of the gather; the trees must equal host-built ones."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(14)
    pts = rng.random((50_001, 3)) * 100
    d = torch.as_tensor(pts, device="cuda")[1:]  # 24-byte offset
    a = otg.Tree("points").create(pts[1:], max_depth=8, max_elements=16)
    b = otg.Tree("points").create(d, max_depth=8, max_elements=16)
    b.sync()
    assert np.array_equal(a.location_keys(), b.location_keys())
    q = rng.random((200, 3)) * 100
    assert_csr_equal(a.knn(q, 5), b.knn(q, 5), "unaligned points")
    c = rng.random((30_001, 3)) * 100
    e = rng.uniform(0.05, 1.0, (30_001, 3))
    boxes = np.concatenate([c - e, c + e], 1).astype(np.float32)
    db = torch.as_tensor(boxes, device="cuda")[1:]
    ta = otg.Tree("boxes", np.float32).create(boxes[1:], max_depth=7, max_elements=16)
    tb = otg.Tree("boxes", np.float32).create(db, max_depth=7, max_elements=16)
    tb.sync()
    assert np.array_equal(ta.collision_self(), tb.collision_self())


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("tol", [0.0, 0.25, -1.0])
def test_frustum_on_plane_boundaries(dtype, tol):
    """Boxes with corners on a grid and axis-aligned or diagonal planes through grid values: many
    box-plane relations are exact ties (projected centre at exactly +-radius), where the FP32 plane
    decision must hand over to the reference's double-accumulated radius."""
    rng = np.random.default_rng(31)
    lo = rng.integers(0, 64, (20000, 3)).astype(np.float64)
    ext = rng.integers(0, 4, (20000, 3)).astype(np.float64)
    boxes = np.concatenate([lo, lo + ext], 1).astype(dtype)
    t = _gpu_tree(boxes, KIND_LOOSE_BOXES, 6, None, 8)
    o = oracle().create(boxes, KIND_LOOSE_BOXES, 6, None, 8)
    planes = np.zeros((48, 6, 4), np.float64)
    for q in range(48):
        a, b = rng.integers(4, 30, 3), rng.integers(34, 60, 3)
        for ax in range(3):
            planes[q, 2 * ax, 0], planes[q, 2 * ax, 1 + ax] = a[ax], 1.0
            planes[q, 2 * ax + 1, 0], planes[q, 2 * ax + 1, 1 + ax] = -b[ax], -1.0
        if q % 3 == 0:  # a diagonal plane through grid points
            planes[q, 0] = [rng.integers(20, 60) / np.sqrt(2.0), 1 / np.sqrt(2.0), 1 / np.sqrt(2.0), 0.0]
    planes = planes.astype(dtype)
    assert_csr_equal(t.frustum_culling(planes, tol=tol)[:2], o.frustum(planes, tol=tol), f"frustum tol={tol}")


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("algo", [otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64])
def test_gpu_plane_queries_match_reference_fixture(name, algo):
    """PlaneSearch and PlanePositiveSegmentation (default and 1% tolerance) against the reference."""
    g = load_golden(name)
    t = _gpu_tree(g["entities"], int(g["kind"]), int(g["max_depth"]), g.get("box"), int(g["max_elem"]))
    pl = g["single_planes"]
    tol = float(g["plane_tol"])
    assert_csr_equal(t.plane_search(pl, algo=algo)[:2], (g["plane_off"], g["plane_ids"]), "plane search")
    assert_csr_equal(t.plane_positive_segmentation(pl, algo=algo)[:2], (g["planepos_off"], g["planepos_ids"]), "plane positive")
    assert_csr_equal(t.plane_search(pl, tol, algo=algo)[:2], (g["planetol_off"], g["planetol_ids"]), "plane search, wide tolerance")
    assert_csr_equal(t.plane_positive_segmentation(pl, tol, algo=algo)[:2], (g["planepostol_off"], g["planepostol_ids"]), "plane positive, wide tol")


def _single_planes(rng, n, scale):
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = rng.random((n, 1)) * scale * 1.4 - 0.2 * scale
    ax = np.arange(n) % 3 == 0  # axis-aligned planes on node faces
    nrm[ax] = np.eye(3)[np.arange(ax.sum()) % 3]
    d[ax] = np.round(d[ax] / (scale / 32)) * (scale / 32)
    return np.concatenate([d, nrm], 1)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("kind", [KIND_POINTS, KIND_LOOSE_BOXES, KIND_BOXES])
def test_plane_queries_random(dtype, kind):
    rng = np.random.default_rng(4242 + kind)
    n = 150_000
    if kind == KIND_POINTS:
        ent = rng.random((n, 3)) * 100
        D, me = 9, 16
    else:
        cen = rng.random((n, 3)) * 100
        half = rng.lognormal(np.log(0.3), 0.6, (n, 3))
        ent = np.concatenate([cen - half, cen + half], 1)
        D, me = 7, 24
    ent = ent.astype(dtype)
    t = _gpu_tree(ent, kind, D, None, me)
    o = oracle().create(ent, kind, D, None, me)
    planes = _single_planes(rng, 300, 100).astype(dtype)
    for tol in (-1.0, 0.25):
        ref_s, ref_p = o.plane_search(planes, tol), o.plane_positive(planes, tol)
        for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
            assert_csr_equal(t.plane_search(planes, tol, algo=algo)[:2], ref_s, f"plane search tol={tol} algo={algo}")
            assert_csr_equal(t.plane_positive_segmentation(planes, tol, algo=algo)[:2], ref_p, f"plane positive tol={tol} algo={algo}")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("kind", [KIND_POINTS, KIND_LOOSE_BOXES, KIND_BOXES])
def test_combined_query_random(dtype, kind):
    """Query<And> / Query<Or> with frustum (crossing flags), range Inside / Overlap and plane
    conditions, batched and plain, against the oracle."""
    from _compare import random_query_program

    rng = np.random.default_rng(777 + kind)
    n = 120_000
    if kind == KIND_POINTS:
        ent = rng.random((n, 3)) * 100
        D, me = 8, 16
    else:
        cen = rng.random((n, 3)) * 100
        half = rng.lognormal(np.log(0.3), 0.6, (n, 3))
        ent = np.concatenate([cen - half, cen + half], 1)
        D, me = 7, 24
    ent = ent.astype(dtype)
    t = _gpu_tree(ent, kind, D, None, me)
    o = oracle().create(ent, kind, D, None, me)
    conds, off, planes, cross, boxes = random_query_program(rng, 200, 100.0, dtype)
    for logical_or in (False, True):
        ref = o.query(conds, off, planes, cross, boxes, or_op=logical_or)
        assert len(ref[1]) > 0
        for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
            got = t.query(conds, off, planes, cross, boxes, logical_or=logical_or, algo=algo)
            assert_csr_equal(got[:2], ref, f"query or={logical_or} algo={algo}")


def test_combined_query_rejects_bad_conditions():
    t = _gpu_tree(np.random.default_rng(1).random((1000, 3)), KIND_POINTS, 4, None, 8)
    bad = np.zeros(1, otg.COND_DTYPE)
    bad["kind"] = otg.COND_PLANE
    bad["first"] = 3  # one plane given
    with pytest.raises(otg.OtgError):
        t.query(bad, [0, 1], np.array([[0.5, 1.0, 0, 0]]), np.zeros(1, np.uint8))
    bad["kind"] = 9
    bad["first"] = 0
    with pytest.raises(otg.OtgError):
        t.query(bad, [0, 1], np.array([[0.5, 1.0, 0, 0]]), np.zeros(1, np.uint8))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("kind", [KIND_POINTS, KIND_LOOSE_BOXES])
@pytest.mark.parametrize("offset", [0, 1])
def test_build_from_pinned_host_memory(kind, dtype, offset):
    """Entities in pinned host memory: the bounding-box pass reads them where they are and writes the
    device copy (offset 1 entity: a source that is not 16-byte aligned; an odd count: a partial last
    chunk). The tree equals the oracle's."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31 + kind + offset)
    n = 100_003
    if kind == KIND_POINTS:
        ent = rng.random((n + offset, 3)) * 100
    else:
        c = rng.random((n + offset, 3)) * 100
        h = rng.random((n + offset, 3))
        ent = np.concatenate([c - h, c + h], 1)
    pinned = torch.from_numpy(ent.astype(dtype)).pin_memory()[offset:]
    host = pinned.numpy()
    t = otg.Tree(GPU_KIND[kind], dtype).create(pinned, max_depth=8, max_elements=16)
    o = oracle().create(host, kind, 8, None, 16)
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal(t.nodes(), o.nodes(), "pinned")
    q = _queries(rng, dtype, 100)
    assert_csr_equal(t.range_search(q["ranges"], 1)[:2], o.range_search(q["ranges"], 1), "pinned range")


@pytest.mark.parametrize("n", [1, 7, 4095, 4096, 4097, 3 * 4096 + 1, 1_000_003])
@pytest.mark.parametrize("kind,depth", [(KIND_POINTS, 10), (KIND_POINTS, 19), (KIND_POINTS, 3), (KIND_LOOSE_BOXES, 12), (KIND_LOOSE_BOXES, 10)])
def test_sort_sizes_and_digit_widths(n, kind, depth):
    """Sizes around the radix sort's 4096-key tiles (one partial tile, exact tiles, a partial last
    tile, chunks of unequal tile counts) and key widths that give 1 to 6 passes of 8-11-bit
    digits (points at depth 3, 10, 19: 10, 31, 58 bits; boxes at depth 10 and 12: 35 and 41
    bits): keys and node sets equal the oracle's."""
    rng = np.random.default_rng(n * 31 + depth)
    if kind == KIND_POINTS:
        ent = rng.random((n, 3)) * 100
        ent[: n // 3] = np.round(ent[: n // 3])  # repeated locations: equal keys keep id order
    else:
        c = rng.random((n, 3)) * 100
        ent = np.concatenate([c - rng.random((n, 3)) * 0.3, c + rng.random((n, 3)) * 0.3], 1)
    t = _gpu_tree(ent, kind, depth, None, 8)
    o = oracle().create(ent, kind, depth, None, 8)
    assert np.array_equal(t.location_keys(), o.location_keys())
    assert_nodes_equal_exact(t.nodes(), o.nodes(), f"n={n} depth={depth}")


@pytest.mark.parametrize("kind", [KIND_POINTS, KIND_LOOSE_BOXES, KIND_BOXES])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("device_span", [False, True])
def test_core_form_set_entities(kind, dtype, device_span):
    """The Core form's entity span (otg_tree_set_entities): a tree created from one span answers with
    another span of the same size as the reference's Core queries do, for the queries that test a
    fixed set of nodes (the oracle pins that against the reference in test_oracle_vs_reference.py),
    then answers every query with a copy of its Create span; a span of another size is refused."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(71 + kind)
    n = 60_000
    if kind == KIND_POINTS:
        ent = (rng.random((n, 3)) * 10).astype(dtype)
    else:
        c = rng.random((n, 3)) * 10
        h = rng.random((n, 3)) * 0.05
        ent = np.concatenate([c - h, c + h], 1).astype(dtype)
    t = _gpu_tree(ent, kind, 8, None, 12)
    o = oracle().create(ent, kind, 8, None, 12)
    qs = _queries(rng, dtype, 10, nq=300)
    new = moved_span(ent, rng, kind != KIND_POINTS)
    # a moved span: the queries that test a fixed set of nodes and entities (where entities left
    # the nodes they were built into, the reference's kNN, first-hit and collision answers depend
    # on the order of its own traversal)
    t.set_entities(torch.as_tensor(new, device="cuda") if device_span else new)
    o.set_entities(new)
    for mode in (0, 1):
        assert_csr_equal(t.range_search(qs["ranges"], mode)[:2], o.range_search(qs["ranges"], mode), f"moved span range{mode}")
    assert_csr_equal(t.pick_search(qs["qpts"])[:2], o.pick_search(qs["qpts"]), "moved span pick")
    assert_csr_equal(t.frustum_culling(qs["planes"])[:2], o.frustum(qs["planes"]), "moved span frustum")
    g = t.ray_all(qs["rays"], tol=0.005)
    r = o.ray(qs["rays"], first=False, tol=0.005)
    assert_csr_equal(g[:2], r[:2], "moved span ray all")
    assert_dist_close(g[2], r[2], RAY_REL, "moved span ray all")
    # the Create span again (a copy: another pointer, the same geometry): every query. The ray
    # tolerance scales with the domain (10 here, 100 in the random tests): with a tolerance near the
    # points' spacing, RayIntersectedFirst's bound can grow back while the reference examines entities,
    # and its answer depends on that order
    t.set_entities(torch.as_tensor(ent.copy(), device="cuda") if device_span else ent.copy())
    o.set_entities(ent)
    _check_queries(t, o, qs, kind, 0.005, f"core span kind={kind}")
    if kind != KIND_POINTS:
        assert np.array_equal(t.collision_self(), o.collide_self())
    with pytest.raises(otg.OtgError):
        t.set_entities(ent[:-1])


@pytest.mark.parametrize("tol", [0.0, -1.0, 1e-9, 0.5])
def test_range_on_exact_boundaries(tol):
    """Points on an integer lattice and one ulp either side of it, ranges whose faces lie on lattice
    values or one ulp off them: the batched kernel's FP32 pre-tests must leave every such case to
    the FP64 test and answer exactly as the reference."""
    rng = np.random.default_rng(31)
    lat = rng.integers(0, 64, (60_000, 3)).astype(np.float64)
    wiggle = rng.integers(-1, 2, lat.shape)
    pts = np.where(wiggle < 0, np.nextafter(lat, -np.inf), np.where(wiggle > 0, np.nextafter(lat, np.inf), lat))
    pts = np.concatenate([pts, lat[:20_000] * 1e-3, lat[:20_000] + 1e6])  # small and large magnitudes
    lo = rng.integers(0, 60, (3000, 3)).astype(np.float64)
    hi = lo + rng.integers(0, 6, (3000, 3))
    lo = np.where(rng.random(lo.shape) < 0.3, np.nextafter(lo, np.inf), lo)
    hi = np.where(rng.random(hi.shape) < 0.3, np.nextafter(hi, -np.inf), hi)
    ranges = np.concatenate([lo, hi], 1)
    ranges = np.concatenate([ranges, ranges[:500] * 1e-3, ranges[:500] + 1e6])
    t = _gpu_tree(pts, KIND_POINTS, 10, None, 8)
    o = oracle().create(pts, KIND_POINTS, 10, None, 8)
    for mode in (0, 1):
        ref = o.range_search(ranges, mode, tol)
        for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
            assert_csr_equal(t.range_search(ranges, mode, tol=tol, algo=algo)[:2], ref, f"range mode {mode} tol {tol} algo {algo}")


@pytest.mark.parametrize("sizes", ["small", "medium", "with_long"])
def test_result_runs_of_every_length(sizes):
    """Results are put in canonical order per query by counting and a sort of each query's run:
    runs of at most 32 ids, runs of 33-1024 ids, and batches holding a longer run (which take the
    radix sort of the whole result instead) all give the oracle's ids."""
    rng = np.random.default_rng({"small": 41, "medium": 42, "with_long": 43}[sizes])
    pts = rng.random((100_000, 3)) * 100
    c = rng.random((400, 3)) * 100
    half = {"small": 1.0, "medium": 5.0, "with_long": 5.0}[sizes] * (0.5 + rng.random((400, 1)))
    if sizes == "with_long":
        half[:3] = 30.0  # tens of thousands of ids each
    ranges = np.concatenate([c - half, c + half], 1)
    t = _gpu_tree(pts, KIND_POINTS, 8, None, 16)
    o = oracle().create(pts, KIND_POINTS, 8, None, 16)
    ref = o.range_search(ranges, 0)
    counts = np.diff(ref[0].astype(np.int64))
    if sizes == "small":
        assert counts.max() <= 32
    elif sizes == "medium":
        assert counts.max() <= 1024 and counts.max() > 32
    else:
        assert counts.max() > 1024
    for algo in (otg.ALGO_DEFAULT, otg.ALGO_PLAIN_FP64):
        assert_csr_equal(t.range_search(ranges, 0, algo=algo)[:2], ref, f"range runs {sizes} algo {algo}")
    planes = np.concatenate([rng.random((50, 1)) * 60 + 20, rng.normal(size=(50, 3))], 1)
    planes[:, 1:] /= np.linalg.norm(planes[:, 1:], axis=1, keepdims=True)
    assert_csr_equal(t.plane_search(planes, tol=0.05)[:2], o.plane_search(planes, 0.05), f"plane runs {sizes}")
