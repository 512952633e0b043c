"""Known-answer cases of the reference's own unit tests, checked against the CPU oracle.

tests/unittests/general.tests.cpp:182-204 (3-D Morton codes), example.tests.cpp:16-38 (Example1,
3-D points), general.tests.cpp:1580-1596 (3-D ray through boxes), and example.tests.cpp:41-90
(Example2). Example2 is a 2-D quadtree case in the reference; here every box is extruded to
z in [0, 1], which leaves each predicate's answer unchanged (all boxes overlap strictly in z).
"""
import numpy as np
import pytest

from _compare import tree_is_equal_to_static
from _oracle_lib import KIND_BOXES, KIND_LOOSE_BOXES, KIND_POINTS, oracle


def _morton(x, y, z):
    # a one-point tree at depth D stores its location in the key: build a 2x2x2 grid and read it
    pts = np.array([[x, y, z], [0, 0, 0], [1, 1, 1]], np.float64)
    t = oracle().create(pts, KIND_POINTS, 1, np.array([0, 0, 0, 2, 2, 2], np.float64), 16)
    return int(t.location_keys()[0]) >> 5


def test_morton_3d_vectors():
    # general.tests.cpp:182-204: {0,0,0}->0, {1,0,0}->1, {0,0,1}->4, {1,1,1}->7
    assert _morton(0.5, 0.5, 0.5) == 0
    assert _morton(1.5, 0.5, 0.5) == 1
    assert _morton(0.5, 0.5, 1.5) == 4
    assert _morton(1.5, 1.5, 1.5) == 7


def test_example1_points():
    pts = np.array([[0, 0, 0], [1, 1, 1], [2, 2, 2]], np.float64)
    t = oracle().create(pts, KIND_POINTS, 3, None, 16)
    off, ids = t.range_search(np.array([[0.5, 0.5, 0.5, 2.5, 2.5, 2.5]]))
    assert sorted(ids.tolist()) == [1, 2]
    off, ids, d = t.knn(np.array([[1.1, 1.1, 1.1]]), 2)
    assert sorted(ids.tolist()) == [1, 2]


def test_ray_3d_general_34():
    boxes = np.array(
        [
            [2.0, 0.0, 1.0, 3.0, 1.0, 2.0],
            [3.0, 1.0, 1.0, 4.0, 2.0, 2.0],
            [3.0, 2.0, 1.0, 4.0, 3.0, 2.0],
            [2.0, 3.0, 1.5, 4.0, 4.0, 2.0],
            [2.5, 2.5, 1.5, 3.5, 3.5, 2.0],
        ]
    )
    s = 1.0 / np.sqrt(3.0)
    t = oracle().create(boxes, KIND_LOOSE_BOXES, 3, None, 2)
    off, ids, d = t.ray(np.array([[2.6, 2.8, 1.0, s, s, s]]), tol=0.0)
    assert sorted(ids.tolist()) == [3, 4]


def _example2_boxes():
    b2 = np.array([[0, 0, 1, 1], [1, 1, 2, 2], [2, 2, 3, 3], [3, 3, 4, 4], [1.2, 1.2, 2.8, 2.8]], np.float64)
    return np.stack([b2[:, 0], b2[:, 1], np.zeros(5), b2[:, 2], b2[:, 3], np.ones(5)], 1)


def test_example2_boxes_extruded():
    boxes = _example2_boxes()
    t = oracle().create(boxes, KIND_LOOSE_BOXES, 3, None, 1)
    assert t.collide_self().tolist() == [[1, 4], [2, 4]]
    rng = np.array([[1.0, 1.0, -1.0, 3.1, 3.1, 2.0]])
    assert sorted(t.range_search(rng, 0)[1].tolist()) == [1, 2, 4]
    assert sorted(t.range_search(rng, 1)[1].tolist()) == [1, 2, 3, 4]
    assert sorted(t.pick_search(np.array([[2.5, 2.5, 0.5]]))[1].tolist()) == [2, 4]


def _dynamic_vs_static_boxes():
    """The entities of DynamicVsStaticTest (tests/unittests/general.tests.cpp:5313-5377): five boxes
    in the domain [0, 10]^3, max depth 10, max 2 elements per node; the modified set moves the first
    box's min x by -1.5."""
    boxes = np.array(
        [
            [1.0, 1.0, 1.0, 2.0, 2.0, 2.0],
            [1.1, 1.1, 1.1, 2.1, 2.1, 2.1],
            [4.5, 4.5, 4.5, 5.5, 5.5, 5.5],
            [8.0, 8.0, 8.0, 9.0, 9.0, 9.0],
            [8.1, 8.1, 8.1, 9.1, 9.1, 9.1],
        ]
    )
    modified = boxes.copy()
    modified[0, 0] -= 1.5
    return boxes, modified, np.array([0.0, 0, 0, 10, 10, 10])


@pytest.mark.parametrize("kind", [KIND_LOOSE_BOXES, KIND_BOXES])
def test_dynamic_vs_static_structure(kind):
    """ComparisonTest_MBR_Loose / _NotLoose (general.tests.cpp:5379-5397): the dynamic and the static
    tree of the five boxes have the same node count and are IsEqualTo each other; the static tree of
    the modified boxes is not equal to the dynamic one."""
    boxes, modified, domain = _dynamic_vs_static_boxes()
    dyn = oracle().create(boxes, kind, 10, domain, 2)
    st = dyn.static_layout()
    assert len(st["depth"]) == dyn.node_count
    tol = float(np.finfo(np.float64).eps * 100)
    assert tree_is_equal_to_static(dyn.nodes(), st, tol)
    st_mod = oracle().create(modified, kind, 10, domain, 2).static_layout()
    assert not tree_is_equal_to_static(dyn.nodes(), st_mod, tol)
