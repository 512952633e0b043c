"""Random seeded cases: the CPU oracle against the reference library itself. Runs only where the
reference harness was built from the reference sources (oracle/_ref); elsewhere it is skipped and
the committed golden fixtures carry the pin."""
import numpy as np
import pytest

from _compare import assert_static_equal, moved_span, space_of, static_archive_bytes, tree_is_equal_to_static
from _oracle_lib import KIND_BOXES, KIND_LOOSE_BOXES, KIND_POINTS, oracle, reference

pytestmark = pytest.mark.skipif(reference() is None, reason="reference harness not built here")


def _same_tree(a, b):
    na, nb = a.nodes(), b.nodes()
    return a.max_depth == b.max_depth and np.array_equal(a.location_keys(), b.location_keys()) and all(np.array_equal(na[k], nb[k]) for k in na)


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_random_points(seed, dtype):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(50, 4000))
    pts = (rng.random((n, 3)) * 100).astype(dtype)
    D = int(rng.integers(0, 9))
    me = int(rng.integers(1, 24))
    a, b = oracle().create(pts, KIND_POINTS, D, None, me), reference().create(pts, KIND_POINTS, D, None, me)
    assert _same_tree(a, b)
    c = rng.random((100, 3)) * 100
    e = rng.random((100, 3)) * 8
    ranges = np.concatenate([c - e, c + e], 1).astype(dtype)
    for x, y in zip(a.range_search(ranges), b.range_search(ranges)):
        assert np.array_equal(x, y)
    q = (rng.random((100, 3)) * 100).astype(dtype)
    k = rng.integers(1, 30, 100).astype(np.uint32)
    for x, y in zip(a.knn(q, k), b.knn(q, k)):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("kind", [KIND_LOOSE_BOXES, KIND_BOXES])
def test_random_boxes(seed, kind):
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(50, 2500))
    cen = rng.random((n, 3)) * 100
    half = rng.random((n, 3)) * 3
    boxes = np.concatenate([cen - half, cen + half], 1)
    D = int(rng.integers(0, 7))
    me = int(rng.integers(1, 20))
    a, b = oracle().create(boxes, kind, D, None, me), reference().create(boxes, kind, D, None, me)
    assert _same_tree(a, b)
    assert np.array_equal(a.collide_self(), b.collide_self())
    assert np.array_equal(b.collide_self(), b.collide_self_par())


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_collision_rounding_gap(dtype):
    """Boxes whose x faces are one ulp apart where the tolerance lies between half an ulp and an ulp
    (coordinates in [140, 200]): the reference's sweep-and-prune decides these pairs."""
    rng = np.random.default_rng(77)
    n = 1500
    cen = rng.random((n, 3)) * 60 + 140
    half = np.round(rng.random((n, 3)) * 4 + 0.5, 1)
    ent = np.concatenate([cen - half, cen + half], 1).astype(dtype)
    ent[n // 2 :, 0] = ent[: n - n // 2, 3]
    ent[n // 2 :, 3] = ent[n // 2 :, 0] + dtype(2.0)
    ent[n // 2 :, 0] = np.nextafter(ent[n // 2 :, 0], dtype(1e9))
    ent[n // 2 :, 3] = np.maximum(ent[n // 2 :, 3], ent[n // 2 :, 0])
    a, b = oracle().create(ent, KIND_LOOSE_BOXES, 4, None, 4), reference().create(ent, KIND_LOOSE_BOXES, 4, None, 4)
    assert np.array_equal(a.collide_self(), b.collide_self())
    other = ent.copy()
    other[:, [0, 3]] = other[:, [0, 3]] + (other[:, 3:4] - other[:, 0:1])
    a2, b2 = oracle().create(other, KIND_LOOSE_BOXES, 4, None, 4), reference().create(other, KIND_LOOSE_BOXES, 4, None, 4)
    assert np.array_equal(a.collide_pair(a2), b.collide_pair(b2))


def _planes(rng, n, scale):
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    # offsets through the data, a share of axis-aligned planes (node faces lie on them exactly)
    d = rng.random((n, 1)) * scale * 1.4 - 0.2 * scale
    ax = rng.random(n) < 0.3
    nrm[ax] = np.eye(3)[rng.integers(0, 3, ax.sum())]
    d[ax] = np.round(d[ax] / (scale / 16)) * (scale / 16)
    return np.concatenate([d, nrm], 1)


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("kind", [KIND_POINTS, KIND_LOOSE_BOXES])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_plane_search_and_segmentation(seed, kind, dtype):
    """PlaneSearch and PlanePositiveSegmentation of the oracle against the reference's."""
    rng = np.random.default_rng(200 + seed)
    n = int(rng.integers(100, 3000))
    if kind == KIND_POINTS:
        ent = rng.random((n, 3)) * 100
    else:
        cen = rng.random((n, 3)) * 100
        half = rng.random((n, 3)) * 2
        ent = np.concatenate([cen - half, cen + half], 1)
    ent = ent.astype(dtype)
    D = int(rng.integers(2, 8))
    me = int(rng.integers(1, 20))
    a, b = oracle().create(ent, kind, D, None, me), reference().create(ent, kind, D, None, me)
    planes = _planes(rng, 120, 100).astype(dtype)
    for tol in (-1.0, 0.5):
        for x, y in zip(a.plane_search(planes, tol), b.plane_search(planes, tol)):
            assert np.array_equal(x, y)
        for x, y in zip(a.plane_positive(planes, tol), b.plane_positive(planes, tol)):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("kind", [KIND_POINTS, KIND_LOOSE_BOXES, KIND_BOXES])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_combined_query(seed, kind, dtype):
    """Query<And> and Query<Or> with frustum, range and plane conditions: oracle against reference."""
    from _compare import random_query_program

    rng = np.random.default_rng(300 + seed)
    n = int(rng.integers(200, 3000))
    if kind == KIND_POINTS:
        ent = rng.random((n, 3)) * 100
    else:
        cen = rng.random((n, 3)) * 100
        half = rng.random((n, 3)) * 2
        ent = np.concatenate([cen - half, cen + half], 1)
    ent = ent.astype(dtype)
    D = int(rng.integers(2, 7))
    me = int(rng.integers(1, 20))
    a, b = oracle().create(ent, kind, D, None, me), reference().create(ent, kind, D, None, me)
    prog = random_query_program(rng, 80, 100.0, dtype)
    for or_op in (False, True):
        for x, y in zip(a.query(*prog, or_op=or_op), b.query(*prog, or_op=or_op)):
            assert np.array_equal(x, y)


def _static_cases():
    rng = np.random.default_rng(77)
    pts = rng.random((4000, 3))
    clustered = np.concatenate([rng.normal(0.5, 0.001, (2500, 3)), rng.random((1500, 3)), np.repeat(rng.random((5, 3)), 40, 0)])
    c = rng.random((3000, 3)) * 100
    h = rng.random((3000, 3)) * 2
    boxes = np.concatenate([c - h, c + h], 1)
    outside = np.concatenate([boxes, [[-50.0, -50, -50, 200, 200, 200], [-5.0, -5, -5, -1, -1, -1]]])
    space = np.array([0.0, 0, 0, 100, 100, 100])
    return {
        "points": (pts, KIND_POINTS, 6, None, 8),
        "points_f32": (pts.astype(np.float32), KIND_POINTS, 6, None, 8),
        "clustered_deep": (clustered, KIND_POINTS, 19, None, 2),
        "clustered_estimated_depth": (clustered, KIND_POINTS, 0, None, 16),
        "max_elem_1": (pts[:900], KIND_POINTS, 8, None, 1),
        "single_leaf": (pts[:10], KIND_POINTS, 6, None, 16),
        "empty": (np.zeros((0, 3)), KIND_POINTS, 4, None, 16),
        # the empty trees of the GPU archive test: a given box instead of the inverted one
        "empty_points_box": (np.zeros((0, 3)), KIND_POINTS, 4, np.array([0.0, 0, 0, 4, 5, 6]), 16),
        "empty_loose_boxes_box": (np.zeros((0, 6)), KIND_LOOSE_BOXES, 4, np.array([1.0, 1, 1, 9, 9, 9]), 16),
        "loose_boxes": (boxes, KIND_LOOSE_BOXES, 7, None, 4),
        "loose_boxes_f32": (boxes.astype(np.float32), KIND_LOOSE_BOXES, 7, None, 4),
        "loose_boxes_outside_space": (outside, KIND_LOOSE_BOXES, 6, space, 3),
        "boxes_outside_space": (outside, KIND_BOXES, 6, space, 3),
        "duplicate_boxes": (np.repeat(boxes[:5], 50, 0), KIND_LOOSE_BOXES, 9, None, 4),
        "loose_boxes_deep": (boxes, KIND_LOOSE_BOXES, 17, None, 2),
    }


@pytest.mark.parametrize("case", list(_static_cases()))
def test_static_layout(case):
    """The oracle's static linear layout against the reference's StaticOctreePoint / StaticOctreeBox
    (parallel Create) of the same entities."""
    ent, kind, depth, box, max_elem = _static_cases()[case]
    got = oracle().create(ent, kind, depth, box, max_elem).static_layout()
    ref = reference().create(ent, kind, depth, box, max_elem).static_layout()
    assert got is not None and ref is not None
    assert_static_equal(got, ref, case)


def test_static_layout_undefined_for_points_outside_space():
    pts = np.random.default_rng(5).random((500, 3))
    box = np.array([0.2, 0.2, 0.2, 0.8, 0.8, 0.8])
    assert oracle().create(pts, KIND_POINTS, 5, box, 4).static_layout() is None
    assert reference().create(pts, KIND_POINTS, 5, box, 4).static_layout() is None


@pytest.mark.parametrize("managed", [False, True])
@pytest.mark.parametrize("case", list(_static_cases()))
def test_static_archive_format(case, managed):
    """The archive writer restated in tests/_compare.py gives the reference's own BinaryOutputArchive
    bytes of its static tree (core, or Managed with the entities), fed with the reference's layout."""
    ent, kind, depth, box, max_elem = _static_cases()[case]
    t = reference().create(ent, kind, depth, box, max_elem)
    is_box = kind != KIND_POINTS
    mn, size = space_of(ent, is_box, box)
    mine = static_archive_bytes(t.static_layout(), is_box, ent.dtype, len(ent), t.max_depth, max_elem, mn, size, ent if managed else None)
    assert mine == t.static_archive(managed)


@pytest.mark.parametrize("case", list(_static_cases()))
def test_reference_loads_oracle_archive(case):
    """Archive bytes of the oracle's layout load into the reference's static tree type, which then
    IsEqualTo the reference's own tree and holds exactly the archived arrays."""
    ent, kind, depth, box, max_elem = _static_cases()[case]
    o = oracle().create(ent, kind, depth, box, max_elem)
    is_box = kind != KIND_POINTS
    mn, size = space_of(ent, is_box, box)
    lay = o.static_layout()
    data = static_archive_bytes(lay, is_box, ent.dtype, len(ent), o.max_depth, max_elem, mn, size, ent)
    loaded = reference().create(ent, kind, depth, box, max_elem).static_load(data)
    assert loaded is not None
    arrays, equal = loaded
    assert equal
    assert_static_equal(arrays, lay, case, exact_storage=True)
    # a cut archive does not load
    assert reference().create(ent, kind, depth, box, max_elem).static_load(data[:-1]) is None


@pytest.mark.parametrize("case", list(_static_cases()))
def test_is_equal_to_restatement(case):
    """tests/_compare.py: tree_is_equal_to_static answers as the reference's own IsEqualTo between
    its dynamic tree and its static tree of the same entities (equal where no node passes its
    entities through, unequal where the static tree contracts such nodes)."""
    ent, kind, depth, box, max_elem = _static_cases()[case]
    r = reference().create(ent, kind, depth, box, max_elem)
    want = r.lib.oro_dynamic_equals_static(r.h)
    assert want in (0, 1)
    tol = float(np.finfo(ent.dtype).eps * 100)
    assert tree_is_equal_to_static(r.nodes(), r.static_layout(), tol) == bool(want)


def _fuzz_case(seed):
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
        h = rng.random((len(c), 3)) * scale * 0.02 + scale * 1e-4  # every box has extent
        ent = np.concatenate([c - h, c + h], 1)
        if rng.random() < 0.3:
            box = np.array([-0.1, -0.1, -0.1, 1.1, 1.1, 1.1]) * scale
    return ent.astype(dtype), kind, depth, box, max_elem


@pytest.mark.parametrize("seed", range(40))
def test_static_fuzz(seed):
    """Random small trees (kind, scalar, depth, max elements, distribution, given box): the oracle's
    static layout, the archive writer and the IsEqualTo restatement against the reference."""
    ent, kind, depth, box, max_elem = _fuzz_case(seed)
    r = reference().create(ent, kind, depth, box, max_elem)
    o = oracle().create(ent, kind, depth, box, max_elem)
    ref = r.static_layout()
    got = o.static_layout()
    assert (ref is None) == (got is None)
    if ref is None:
        return
    assert_static_equal(got, ref, f"fuzz {seed}")
    is_box = kind != KIND_POINTS
    mn, size = space_of(ent, is_box, box)
    assert static_archive_bytes(ref, is_box, ent.dtype, len(ent), r.max_depth, max_elem, mn, size, ent) == r.static_archive(True)
    tol = float(np.finfo(ent.dtype).eps * 100)
    assert tree_is_equal_to_static(r.nodes(), ref, tol) == bool(r.lib.oro_dynamic_equals_static(r.h))


@pytest.mark.parametrize("kind", [KIND_POINTS, KIND_LOOSE_BOXES, KIND_BOXES])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_core_form_queries_with_another_span(kind, dtype):
    """The Core form: a tree created from one span answers queries with another span of the same
    size (set_entities) as the reference's Core queries answer with the span they are given; the
    oracle restatement equals the reference on every query kind."""
    rng = np.random.default_rng(61 + kind)
    n = 3000
    if kind == KIND_POINTS:
        ent = (rng.random((n, 3)) * 10).astype(dtype)
    else:
        c = rng.random((n, 3)) * 10
        h = rng.random((n, 3)) * 0.2
        ent = np.concatenate([c - h, c + h], 1).astype(dtype)
    o = oracle().create(ent, kind, 6, None, 8)
    r = reference().create(ent, kind, 6, None, 8)
    new = moved_span(ent, rng, kind != KIND_POINTS)
    o.set_entities(new)
    r.set_entities(new)
    c = rng.random((80, 3)) * 10
    e = rng.random((80, 3)) * 1.5
    ranges = np.concatenate([c - e, c + e], 1).astype(dtype)
    for mode in (0, 1):
        for x, y in zip(o.range_search(ranges, mode), r.range_search(ranges, mode)):
            assert np.array_equal(x, y)
    q = (rng.random((80, 3)) * 10).astype(dtype)
    for x, y in zip(o.knn(q, 6), r.knn(q, 6)):
        assert np.array_equal(x, y)
    for x, y in zip(o.pick_search(q), r.pick_search(q)):
        assert np.array_equal(x, y)
    if kind != KIND_POINTS:
        assert np.array_equal(o.collide_self(), r.collide_self())
