"""The CPU oracle (oracle/otg_oracle.hpp) against the golden fixtures produced by the reference
itself (tests/golden/make_golden.py). This pins the restatement to the reference."""
import numpy as np
import pytest

from _compare import (
    assert_csr_equal,
    assert_static_equal,
    golden_cases,
    load_golden,
    node_dict,
    space_of,
    static_archive_bytes,
    static_from_golden,
)
from _oracle_lib import KIND_POINTS, oracle


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_fixture(name):
    g = load_golden(name)
    kind = int(g["kind"])
    t = oracle().create(g["entities"], kind, int(g["max_depth"]), g.get("box"), int(g["max_elem"]))
    assert t.max_depth == int(g["depth"])
    assert np.array_equal(t.location_keys(), g["loc"])
    nd = t.nodes()
    ref = node_dict("node_", g)
    for k in ("keys", "min", "size", "eoff", "eids"):
        assert np.array_equal(nd[k], ref[k]), f"node field {k}"
    for mode in (0, 1):
        assert_csr_equal(t.range_search(g["ranges"], mode), (g[f"range{mode}_off"], g[f"range{mode}_ids"]), f"range{mode}")
    assert_csr_equal(t.pick_search(g["qpts"]), (g["pick_off"], g["pick_ids"]), "pick")
    assert_csr_equal(t.knn(g["qpts"], g["k"]), (g["knn_off"], g["knn_ids"], g["knn_dist"]), "knn")
    assert_csr_equal(t.frustum(g["planes"]), (g["frustum_off"], g["frustum_ids"]), "frustum")
    for first in (0, 1):
        assert_csr_equal(
            t.ray(g["rays"], first=bool(first), tol=float(g["ray_tol"])), (g[f"ray{first}_off"], g[f"ray{first}_ids"], g[f"ray{first}_dist"]), f"ray{first}"
        )
    if kind != KIND_POINTS:
        assert np.array_equal(t.collide_self(), g["collide"])
        t2 = oracle().create(g["other"], kind, int(g["max_depth"]), None, int(g["max_elem"]))
        assert np.array_equal(t.collide_pair(t2), g["collide_pair"])


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_plane_queries_match_reference_fixture(name):
    """PlaneSearch and PlanePositiveSegmentation (default and 1% tolerance) against the reference."""
    g = load_golden(name)
    t = oracle().create(g["entities"], int(g["kind"]), int(g["max_depth"]), g.get("box"), int(g["max_elem"]))
    pl = g["single_planes"]
    assert_csr_equal(t.plane_search(pl), (g["plane_off"], g["plane_ids"]), "plane search")
    assert_csr_equal(t.plane_positive(pl), (g["planepos_off"], g["planepos_ids"]), "plane positive")
    tol = float(g["plane_tol"])
    assert_csr_equal(t.plane_search(pl, tol), (g["planetol_off"], g["planetol_ids"]), "plane search, wide tolerance")
    assert_csr_equal(t.plane_positive(pl, tol), (g["planepostol_off"], g["planepostol_ids"]), "plane positive, wide tolerance")


@pytest.mark.parametrize("kind", [KIND_POINTS, 1])
def test_threaded_oracle_create_matches_sequential(kind):
    """The oracle's threaded location transform and sort (the reference's ParExec steps, used for
    the timed CPU baseline) build the same tree as its sequential path."""
    rng = np.random.default_rng(12)
    n = 60_000
    if kind == KIND_POINTS:
        ent = rng.random((n, 3)) * 100
    else:
        c = rng.random((n, 3)) * 100
        h = rng.random((n, 3))
        ent = np.concatenate([c - h, c + h], 1)
    a = oracle().create(ent, kind, 8, None, 12)
    b = oracle().create(ent, kind, 8, None, 12, threads=7)
    assert np.array_equal(a.location_keys(), b.location_keys())
    na, nb = a.nodes(), b.nodes()
    for k in na:
        assert np.array_equal(na[k], nb[k]), k


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_static_layout_matches_reference_fixture(name):
    """The static linear layout (StaticLinearOrthoTreeCore's arrays) of the same entities."""
    g = load_golden(name)
    t = oracle().create(g["entities"], int(g["kind"]), int(g["max_depth"]), g.get("box"), int(g["max_elem"]))
    ref = static_from_golden(g)
    got = t.static_layout()
    if ref is None:
        assert got is None
        return
    assert_static_equal(got, ref, name)


@pytest.mark.parametrize("name", golden_cases())
def test_archive_writer_matches_reference_fixture(name):
    """The archive writer restated in tests/_compare.py, fed with the reference's static layout,
    gives the bytes the reference's BinaryOutputArchive wrote for its StaticOctreePointM / BoxM."""
    g = load_golden(name)
    if not int(g["static_defined"]):
        pytest.skip("no static tree for points outside the space")
    ent = g["entities"]
    is_box = int(g["kind"]) != KIND_POINTS
    mn, size = space_of(ent, is_box, g.get("box"))
    data = static_archive_bytes(static_from_golden(g), is_box, ent.dtype, len(ent), int(g["depth"]), int(g["max_elem"]), mn, size, ent)
    assert data == g["static_archive"].tobytes()
