"""Generates the golden fixtures in this folder by running the REFERENCE library itself
(oracle/_ref/libref_orthotree.so, compiled from the reference headers by `make -C oracle ref`)
on small seeded inputs. Each fixture stores the inputs and the reference's canonicalised outputs;
tests/test_golden.py checks the CPU oracle against them and tests/test_gpu_parity.py checks the
GPU path. Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from _oracle_lib import KIND_BOXES, KIND_LOOSE_BOXES, KIND_POINTS, reference  # noqa: E402


def queries(rng, dtype, scale, nq=48):
    c = rng.random((nq, 3)) * scale * 1.1 - 0.05 * scale
    e = rng.random((nq, 3)) * 0.12 * scale
    ranges = np.concatenate([c - e, c + e], 1).astype(dtype)
    pts = (rng.random((nq, 3)) * scale).astype(dtype)
    k = rng.integers(1, 17, nq).astype(np.uint32)
    nrm = rng.normal(size=(6, 6, 3))
    nrm /= np.linalg.norm(nrm, axis=2, keepdims=True)
    planes = np.concatenate([rng.random((6, 6, 1)) * scale * 0.6 - 0.3 * scale, nrm], 2).astype(dtype)
    dirs = rng.normal(size=(nq, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    rays = np.concatenate([rng.random((nq, 3)) * scale, dirs], 1).astype(dtype)
    return dict(ranges=ranges, qpts=pts, k=k, planes=planes, rays=rays)


def run_case(name, ent, kind, max_depth, box, max_elem, q, ray_tol):
    R = reference()
    t = R.create(ent, kind, max_depth, box, max_elem)
    out = dict(entities=ent, kind=np.int32(kind), max_depth=np.uint32(max_depth), max_elem=np.uint64(max_elem), ray_tol=np.float64(ray_tol))
    if box is not None:
        out["box"] = box
    out.update(q)
    out["depth"] = np.uint32(t.max_depth)
    out["loc"] = t.location_keys()
    nd = t.nodes()
    for k, v in nd.items():
        out["node_" + k] = v
    for mode in (0, 1):
        o, i = t.range_search(q["ranges"], mode)
        out[f"range{mode}_off"], out[f"range{mode}_ids"] = o, i
    o, i = t.pick_search(q["qpts"])
    out["pick_off"], out["pick_ids"] = o, i
    o, i, d = t.knn(q["qpts"], q["k"])
    out["knn_off"], out["knn_ids"], out["knn_dist"] = o, i, d
    o, i = t.frustum(q["planes"])
    out["frustum_off"], out["frustum_ids"] = o, i
    # single planes for PlaneSearch / PlanePositiveSegmentation, from their own seed so that the
    # earlier queries of every case stay as they were
    prng = np.random.default_rng(sum(map(ord, name)))
    scale = float(np.max(np.abs(ent))) if ent.size else 1.0
    nrm = prng.normal(size=(48, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    dist = prng.random((48, 1)) * scale * 1.2 - 0.1 * scale
    ax = np.arange(48) % 4 == 0
    nrm[ax] = np.eye(3)[np.arange(ax.sum()) % 3]
    dist[ax] = np.round(dist[ax] / (scale / 8)) * (scale / 8)
    out["single_planes"] = np.concatenate([dist, nrm], 1).astype(ent.dtype)
    o, i = t.plane_search(out["single_planes"])
    out["plane_off"], out["plane_ids"] = o, i
    o, i = t.plane_positive(out["single_planes"])
    out["planepos_off"], out["planepos_ids"] = o, i
    # a wide tolerance (1% of the extent), where points near the plane count as hit
    out["plane_tol"] = np.float64(0.01 * scale)
    o, i = t.plane_search(out["single_planes"], float(out["plane_tol"]))
    out["planetol_off"], out["planetol_ids"] = o, i
    o, i = t.plane_positive(out["single_planes"], float(out["plane_tol"]))
    out["planepostol_off"], out["planepostol_ids"] = o, i
    for first in (0, 1):
        o, i, d = t.ray(q["rays"], first=bool(first), tol=ray_tol)
        out[f"ray{first}_off"], out[f"ray{first}_ids"], out[f"ray{first}_dist"] = o, i, d
    if kind != KIND_POINTS:
        out["collide"] = t.collide_self()
        other = ent.copy()
        other[:, :3] += ent.dtype.type(0.37)
        other[:, 3:] += ent.dtype.type(0.37)
        t2 = R.create(other, kind, max_depth, None, max_elem)
        out["other"] = other
        out["collide_pair"] = t.collide_pair(t2)
    # the reference's static linear tree of the same entities (StaticOctreePoint / StaticOctreeBox,
    # parallel Create); undefined for point trees holding points outside their space
    st = t.static_layout()
    out["static_defined"] = np.int32(st is not None)
    if st is not None:
        for k, v in st.items():
            out["static_" + k] = v
        # the reference's binary archive of its Managed static tree (StaticOctreePointM / BoxM)
        out["static_archive"] = np.frombuffer(t.static_archive(True), np.uint8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "nodes", len(nd["keys"]), "depth", t.max_depth)


def main():
    if reference() is None:
        raise SystemExit("reference harness missing: run `make -C oracle ref` first")
    rng = np.random.default_rng(20261203)
    # OctreePoint, double, bounding box of the data
    pts = rng.random((3000, 3)) * 100
    run_case("points_f64", pts, KIND_POINTS, 6, None, 20, queries(rng, np.float64, 100), 0.4)
    # OctreePoint, double, estimated depth, a given box that leaves entities outside (stored in the root)
    box = np.array([10.0, 5.0, 0.0, 80.0, 95.0, 70.0])
    run_case("points_f64_box", pts, KIND_POINTS, 0, box, 8, queries(rng, np.float64, 100), 0.4)
    # duplicates and grid-aligned values
    dup = np.repeat(np.round(rng.random((150, 3)) * 20), 8, axis=0)
    run_case("points_f64_dups", dup, KIND_POINTS, 4, None, 5, queries(rng, np.float64, 20), 0.2)
    # OctreePoint, float, depth 16 (rasterised in double)
    ptsf = (rng.random((3000, 3)) * 50).astype(np.float32)
    run_case("points_f32_d16", ptsf, KIND_POINTS, 16, None, 12, queries(rng, np.float32, 50), 0.4)
    # OctreeBox (loose), double
    cen = rng.random((2000, 3)) * 100
    half = rng.lognormal(np.log(1.5), 0.6, (2000, 3))
    boxes = np.concatenate([cen - half, cen + half], 1)
    run_case("boxes_f64", boxes, KIND_LOOSE_BOXES, 5, None, 16, queries(rng, np.float64, 100), 0.0)
    # OctreeBox (loose), float
    run_case("boxes_f32", boxes.astype(np.float32), KIND_LOOSE_BOXES, 4, None, 10, queries(rng, np.float32, 100), 0.0)
    # degenerate boxes (points as boxes), given box
    deg = np.concatenate([cen[:600], cen[:600]], 1)
    run_case("boxes_f64_degenerate", deg, KIND_LOOSE_BOXES, 6, np.array([0.0, 0, 0, 100, 100, 100]), 8, queries(rng, np.float64, 100), 0.0)
    # regular (non-loose) box trees, OctreeBoxs<false>: FP64 with the data's bounding box, and FP32
    # in a given box with corners on cell boundaries and boxes outside it (drawn from their own seed,
    # so the earlier cases stay as they were). Every box has extent: the reference asserts on a
    # degenerate box on the max face of its space (si_grid.h:213), where the second tree of the
    # fixture, in its data's bounding box, would have one.
    rrng = np.random.default_rng(20261204)
    run_case("boxes_regular_f64", boxes, KIND_BOXES, 5, None, 16, queries(rrng, np.float64, 100), 0.0)
    grid = np.floor(rrng.random((1200, 3)) * 32) * (100 / 32)
    on_grid = np.concatenate([grid, grid + rrng.integers(1, 3, (1200, 3)) * (100 / 32)], 1)
    on_grid[:20] += 150.0
    run_case("boxes_regular_f32_box", on_grid.astype(np.float32), KIND_BOXES, 6, np.array([0.0, 0, 0, 100, 100, 100], np.float32), 8,
             queries(rrng, np.float32, 100), 0.0)


if __name__ == "__main__":
    main()
