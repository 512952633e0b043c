"""Export to the static linear layout (otg_tree_export_static) and the binary archive of that static
tree (otg_tree_save_static / otg_tree_load_static): the GPU-built tree in the arrays of the
reference's StaticLinearOrthoTreeCore, against the reference's own static trees (golden
fixtures) and the CPU oracle's restatement on seeded inputs, with the refusals where the reference
has no such tree. Child segment begins, entity segments, depth ids and node geometry are compared
bit for bit; entity storage exactly against the oracle (both keep equal locations in id order) and
per node as sets against the reference (its unstable sort leaves that order unspecified)."""
import numpy as np
import pytest

import octree_gb300 as otg
from _compare import (
    GPU_KIND,
    assert_csr_equal,
    assert_static_equal,
    golden_cases,
    load_golden,
    space_of,
    static_archive_bytes,
    static_from_golden,
    tree_is_equal_to_static,
)
from _oracle_lib import KIND_BOXES, KIND_LOOSE_BOXES, KIND_POINTS, oracle

pytestmark = pytest.mark.gpu


def _gpu_tree(ent, kind, max_depth, box, max_elem):
    t = otg.Tree(GPU_KIND[kind], ent.dtype)
    return t.create(ent, max_depth=max_depth, box=box, max_elements=max_elem)


@pytest.mark.parametrize("name", golden_cases())
def test_static_layout_matches_reference_fixture(name):
    g = load_golden(name)
    kind = int(g["kind"])
    t = _gpu_tree(g["entities"], kind, int(g["max_depth"]), g.get("box"), int(g["max_elem"]))
    ref = static_from_golden(g)
    if ref is None:
        with pytest.raises(otg.OtgError):
            t.export_static()
        return
    assert_static_equal(t.export_static(), ref, name)


def _cases():
    rng = np.random.default_rng(2026)
    pts = rng.random((20000, 3)) * 100
    clustered = np.concatenate(
        [rng.normal(50, 0.01, (12000, 3)), rng.random((8000, 3)) * 100, np.repeat(rng.random((20, 3)) * 100, 60, 0)]
    )
    c = rng.random((15000, 3)) * 100
    h = rng.lognormal(np.log(0.8), 0.7, (15000, 3))
    boxes = np.concatenate([c - h, c + h], 1)
    big = np.array([[-50.0, -50, -50, 200, 200, 200], [1.0, 1, 1, 99, 99, 99]])
    space = np.array([0.0, 0, 0, 100, 100, 100])
    return {
        "points": (pts, KIND_POINTS, 8, None, 16),
        "points_f32": (pts.astype(np.float32), KIND_POINTS, 8, None, 16),
        "points_keys64": (clustered, KIND_POINTS, 19, None, 4),
        "clustered_estimated_depth": (clustered, KIND_POINTS, 0, None, 20),
        "max_elem_1": (pts[:3000], KIND_POINTS, 10, None, 1),
        "root_leaf": (pts[:7], KIND_POINTS, 6, None, 16),
        "depth_0": (pts[:300], KIND_POINTS, 1, None, 16),
        "duplicates": (np.repeat(pts[:40], 30, 0), KIND_POINTS, 10, None, 8),
        "boxes": (boxes, KIND_LOOSE_BOXES, 8, None, 8),
        "boxes_f32": (boxes.astype(np.float32), KIND_LOOSE_BOXES, 8, None, 8),
        "boxes_deep": (boxes, KIND_LOOSE_BOXES, 17, None, 2),
        "boxes_outside_space": (np.concatenate([boxes, big]), KIND_LOOSE_BOXES, 6, space, 4),
        "duplicate_boxes": (np.repeat(boxes[:30], 40, 0), KIND_LOOSE_BOXES, 12, None, 6),
        "regular_boxes": (boxes, KIND_BOXES, 8, None, 8),
        "regular_boxes_f32_outside_space": (np.concatenate([boxes, big]).astype(np.float32), KIND_BOXES, 6, space, 4),
    }


@pytest.mark.parametrize("case", list(_cases()))
def test_static_layout_matches_oracle(case):
    ent, kind, depth, box, max_elem = _cases()[case]
    t = _gpu_tree(ent, kind, depth, box, max_elem)
    ref = oracle().create(ent, kind, depth, box, max_elem).static_layout()
    assert ref is not None
    got = t.export_static()
    assert_static_equal(got, ref, case, exact_storage=True)
    # the exported geometry is in the tree's own scalar type
    assert got["geometry"].dtype == ent.dtype


def test_static_layout_empty_tree():
    t = _gpu_tree(np.zeros((0, 3)), KIND_POINTS, 4, None, 16)
    s = t.export_static()
    assert s["child_begins"].size == 0 and s["segments"].shape == (0, 2) and s["depth"].size == 0 and s["entity_storage"].size == 0


def test_static_layout_refusals():
    rng = np.random.default_rng(3)
    pts = rng.random((2000, 3))
    # points outside the given space: the reference's static Build does not end on them
    t = _gpu_tree(pts, KIND_POINTS, 5, np.array([0.2, 0.2, 0.2, 0.8, 0.8, 0.8]), 4)
    with pytest.raises(otg.OtgError):
        t.export_static()
    # a forest has no single static layout
    f = otg.Forest("points").create(pts, np.array([0, 1000, 2000], np.uint64))
    with pytest.raises(otg.OtgError):
        f.export_static()
    # the tree stays usable after a refusal
    assert t.range_search(np.array([[0.0, 0, 0, 1, 1, 1]]))[1].size == 2000


def test_static_layout_full_size_properties():
    """16M clustered points (depth 10, max 20): the layout is a tree over all entities, numbered
    breadth first with children in location order, and equals the oracle on a 2M-point sample."""
    rng = np.random.default_rng(301)
    n = 16_000_000
    pts = np.concatenate([rng.random((int(n * 0.7), 3)), rng.normal(0.5, 0.05, (n - int(n * 0.7), 3))])
    t = _gpu_tree(pts, KIND_POINTS, 10, None, 20)
    s = t.export_static()
    m = s["depth"].size
    cb = s["child_begins_full"]
    seg = s["segments"].astype(np.int64)
    # every entity in exactly one segment
    assert seg[:, 1].sum() == n
    assert np.array_equal(np.sort(s["entity_storage"]), np.arange(n, dtype=np.uint32))
    # child segments: contiguous, in id order, covering nodes 1..m-1 once
    assert cb[0] == 1 and cb[-1] == m and np.all(np.diff(cb.astype(np.int64)) >= 0)
    cnt = np.diff(cb.astype(np.int64))
    parent = np.repeat(np.arange(m), cnt)
    assert parent.size == m - 1
    child = np.arange(1, m)
    # children are deeper than their parent, and their ranges follow the parent's own entities
    assert np.all(s["depth"][child] > s["depth"][parent])
    assert np.all(seg[child, 0] >= seg[parent, 0] + seg[parent, 1])
    # siblings in location order: entity segment begins increase along each child segment
    same = parent[1:] == parent[:-1]
    assert np.all(seg[child[1:], 0][same] > seg[child[:-1], 0][same])
    # a node with children is not a pass-through: two or more children, or entities of its own
    has = cnt > 0
    assert np.all((cnt[has] >= 2) | (seg[has, 1] > 0) | (np.arange(m)[has] == 0))
    sample = pts[:2_000_000]
    ts = _gpu_tree(sample, KIND_POINTS, 10, None, 20)
    assert_static_equal(ts.export_static(), oracle().create(sample, KIND_POINTS, 10, None, 20).static_layout(), "2M sample", exact_storage=True)


# ---------------------------------------------------------------- binary archive (save / resume)


def _writer_bytes(t, lay, ent, kind, box, max_elem, with_entities):
    is_box = kind != KIND_POINTS
    mn, size = space_of(ent, is_box, box)
    return static_archive_bytes(lay, is_box, ent.dtype, len(ent), t.max_depth, max_elem, mn, size, ent if with_entities else None)


@pytest.mark.parametrize("name", golden_cases())
def test_archive_matches_reference_fixture(name):
    """otg_tree_save_static writes the bytes of the reference's BinaryOutputArchive: equal to the
    reference's own archive where both order the entities of every node alike, and always equal to
    the writer restated in tests/_compare.py over the exported layout."""
    g = load_golden(name)
    if not int(g["static_defined"]):
        pytest.skip("no static tree for points outside the space")
    ent, kind, box, me = g["entities"], int(g["kind"]), g.get("box"), int(g["max_elem"])
    t = _gpu_tree(ent, kind, int(g["max_depth"]), box, me)
    lay = t.export_static()
    managed = t.save_static(True)
    assert managed == _writer_bytes(t, lay, ent, kind, box, me, True)
    assert t.save_static(False) == _writer_bytes(t, lay, ent, kind, box, me, False)
    if np.array_equal(lay["entity_storage"], g["static_entity_storage"]):
        assert managed == g["static_archive"].tobytes()


@pytest.mark.parametrize("name", golden_cases())
def test_resume_from_reference_archive(name):
    """A tree resumed from the reference's own archive is the reference's tree: its static layout
    equals the archived one and it answers the fixture's queries as the reference did."""
    g = load_golden(name)
    if not int(g["static_defined"]):
        pytest.skip("no static tree for points outside the space")
    ent, kind = g["entities"], int(g["kind"])
    t = otg.Tree(GPU_KIND[kind], ent.dtype).load_static(g["static_archive"].tobytes(), box=g.get("box"))
    assert_static_equal(t.export_static(), static_from_golden(g), name)
    for mode in (0, 1):
        assert_csr_equal(t.range_search(g["ranges"], mode)[:2], (g[f"range{mode}_off"], g[f"range{mode}_ids"]), f"{name} range{mode}")
    assert_csr_equal(t.knn(g["qpts"], g["k"]), (g["knn_off"], g["knn_ids"], g["knn_dist"]), f"{name} knn")


@pytest.mark.parametrize("case", ["clustered_estimated_depth", "boxes_f32", "duplicate_boxes", "points_keys64", "regular_boxes"])
def test_archive_round_trip(case):
    """save -> resume into a new tree -> save gives the same bytes; the resumed tree is the tree."""
    ent, kind, depth, box, me = _cases()[case]
    t = _gpu_tree(ent, kind, depth, box, me)
    data = t.save_static(True)
    t2 = otg.Tree(GPU_KIND[kind], ent.dtype).load_static(data, box=box)
    assert t2.save_static(True) == data
    assert t2.node_count == t.node_count


def test_resume_refusals():
    rng = np.random.default_rng(9)
    pts = rng.random((5000, 3)) * 10
    t = _gpu_tree(pts, KIND_POINTS, 6, None, 8)
    data = t.save_static(True)
    fresh = lambda dtype=np.float64: otg.Tree("points", dtype)
    with pytest.raises(otg.OtgError):  # the core form holds no entities to rebuild
        fresh().load_static(t.save_static(False))
    with pytest.raises(otg.OtgError):  # cut short
        fresh().load_static(data[:-3])
    with pytest.raises(otg.OtgError):  # trailing bytes
        fresh().load_static(data + b"\0")
    with pytest.raises(otg.OtgError):  # another scalar type
        fresh(np.float32).load_static(data)
    with pytest.raises(otg.OtgError):  # another kind
        otg.Tree("boxes").load_static(data)
    with pytest.raises(otg.OtgError):  # not an archive
        fresh().load_static(bytes(range(256)) * 4)
    # a tree created in a given box does not resume without it (the rebuild differs)
    box = np.array([-1.0, -1, -1, 12, 12, 12])
    tb = _gpu_tree(pts, KIND_POINTS, 6, box, 8)
    with pytest.raises(otg.OtgError):
        fresh().load_static(tb.save_static(True))
    assert fresh().load_static(tb.save_static(True), box=box).save_static(True) == tb.save_static(True)


def test_archive_of_a_tree_built_from_device_memory():
    """A tree built from device memory (read in place, no input-order copy kept) archives the same
    entities and bytes as one built from host memory."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(44)
    c = rng.random((30000, 3)) * 50
    h = rng.random((30000, 3))
    boxes = np.concatenate([c - h, c + h], 1)
    th = _gpu_tree(boxes, KIND_LOOSE_BOXES, 7, None, 8)
    dev = torch.as_tensor(boxes, device="cuda")
    td = otg.Tree("boxes").create(dev, max_depth=7, max_elements=8)
    torch.cuda.synchronize()
    dev.fill_(0.0)  # the archive must not read the caller's array
    torch.cuda.synchronize()
    assert td.save_static(True) == th.save_static(True)


@pytest.mark.parametrize("kind", [KIND_LOOSE_BOXES, KIND_BOXES])
def test_dynamic_vs_static_known_answer(kind):
    """DynamicVsStaticTest (tests/unittests/general.tests.cpp:5313-5397) on the GPU trees: the GPU
    tree and its static export of the five boxes have the same node count and are IsEqualTo each
    other (tests/_compare.py restates IsEqualTo); the export of the modified boxes is not."""
    boxes = np.array(
        [
            [1.0, 1.0, 1.0, 2.0, 2.0, 2.0],
            [1.1, 1.1, 1.1, 2.1, 2.1, 2.1],
            [4.5, 4.5, 4.5, 5.5, 5.5, 5.5],
            [8.0, 8.0, 8.0, 9.0, 9.0, 9.0],
            [8.1, 8.1, 8.1, 9.1, 9.1, 9.1],
        ]
    )
    domain = np.array([0.0, 0, 0, 10, 10, 10])
    t = _gpu_tree(boxes, kind, 10, domain, 2)
    st = t.export_static()
    tol = float(np.finfo(np.float64).eps * 100)
    assert len(st["depth"]) == t.node_count
    assert tree_is_equal_to_static(t.nodes(), st, tol)
    modified = boxes.copy()
    modified[0, 0] -= 1.5
    assert not tree_is_equal_to_static(t.nodes(), _gpu_tree(modified, kind, 10, domain, 2).export_static(), tol)


@pytest.mark.parametrize("case", ["points", "clustered_estimated_depth", "boxes", "regular_boxes", "duplicate_boxes"])
def test_is_equal_to_matches_oracle(case):
    """IsEqualTo between the GPU tree and its static export answers as it does for the oracle's."""
    ent, kind, depth, box, me = _cases()[case]
    tol = float(np.finfo(ent.dtype).eps * 100)
    t = _gpu_tree(ent, kind, depth, box, me)
    o = oracle().create(ent, kind, depth, box, me)
    assert tree_is_equal_to_static(t.nodes(), t.export_static(), tol) == tree_is_equal_to_static(o.nodes(), o.static_layout(), tol)


def _fuzz_case(seed):
    # the random small trees of tests/test_oracle_vs_reference.py: test_static_fuzz (same seeds)
    rng = np.random.default_rng(1000 + seed)
    kind = int(rng.integers(0, 3))
    dtype = np.float64 if rng.random() < 0.6 else np.float32
    n = int(rng.integers(1, 3000))
    depth = int(rng.integers(1, 13)) if rng.random() < 0.8 else 0
    max_elem = int(rng.integers(1, 33))
    scale = 10.0 ** rng.uniform(-2, 3)
    style = rng.integers(0, 3)
    if style == 0:
        c = rng.random((n, 3))
    elif style == 1:
        c = np.clip(rng.normal(0.5, 0.02, (n, 3)), 0, 1)
    else:
        c = np.repeat(rng.random((max(1, n // 20), 3)), 20, 0)[:n]
    c = c * scale
    box = None
    if kind == KIND_POINTS:
        ent = c
    else:
        h = rng.random((len(c), 3)) * scale * 0.02 + scale * 1e-4
        ent = np.concatenate([c - h, c + h], 1)
        if rng.random() < 0.3:
            box = np.array([-0.1, -0.1, -0.1, 1.1, 1.1, 1.1]) * scale
    return ent.astype(dtype), kind, depth, box, max_elem


@pytest.mark.parametrize("seed", range(40))
def test_static_fuzz(seed):
    """Random small trees: the GPU's static layout equals the oracle's (entity order included) and its
    archive equals the writer's bytes."""
    ent, kind, depth, box, max_elem = _fuzz_case(seed)
    t = _gpu_tree(ent, kind, depth, box, max_elem)
    lay = t.export_static()
    assert_static_equal(lay, oracle().create(ent, kind, depth, box, max_elem).static_layout(), f"fuzz {seed}", exact_storage=True)
    assert t.save_static(True) == _writer_bytes(t, lay, ent, kind, box, max_elem, True)


@pytest.mark.parametrize("kind,box", [(KIND_POINTS, None), (KIND_POINTS, [0.0, 0, 0, 4, 5, 6]), (KIND_LOOSE_BOXES, [1.0, 1, 1, 9, 9, 9])])
def test_archive_of_an_empty_tree(kind, box):
    """A Create of no entities still writes the base fields of its space (the given box, or the
    inverted bounding box of nothing) and empty arrays, as the reference's archive holds them (the
    writer's bytes for these three trees are pinned against the reference's own archives in
    test_static_archive_format: cases empty, empty_points_box, empty_loose_boxes_box). The Managed
    archive resumes into a tree that writes the same bytes again."""
    ent = np.zeros((0, 3 if kind == KIND_POINTS else 6))
    b = None if box is None else np.array(box)
    t = _gpu_tree(ent, kind, 4, b, 16)
    data = t.save_static(True)
    assert data == _writer_bytes(t, t.export_static(), ent, kind, b, 16, True)
    assert t.save_static(False) == _writer_bytes(t, t.export_static(), ent, kind, b, 16, False)
    resumed = otg.Tree(GPU_KIND[kind]).load_static(data, box=b)
    assert resumed.save_static(True) == data
