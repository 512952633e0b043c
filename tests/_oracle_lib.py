"""ctypes access to the CPU oracle (oracle/otg_oracle_capi.cpp) and, where it was built, to the
reference harness (oracle/_ref/libref_orthotree.so). Both export the same C-ABI, so every test can
run the same call against either library. Test infrastructure only."""
import ctypes as C
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libotg_oracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libref_orthotree.so")

KIND_POINTS, KIND_LOOSE_BOXES, KIND_BOXES = 0, 1, 2
# one condition of a combined query (the otg_condition record of include/octree_gb300.h)
COND_DTYPE = np.dtype([("kind", "<i4"), ("first", "<u4"), ("count", "<u4"), ("reserved", "<u4"), ("tol", "<f8")])
COND_FRUSTUM, COND_RANGE_INSIDE, COND_RANGE_OVERLAP, COND_PLANE = 0, 1, 2, 3

_vp = C.c_void_p
_u64 = C.c_uint64
_u32 = C.c_uint32
_dbl = C.c_double
_int = C.c_int


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


class OracleLib:
    def __init__(self, path):
        self.path = path
        lib = C.CDLL(path)
        sig = {
            "oro_create": (_vp, [_int, _int, _vp, _u64, _u32, _vp, _u64]),
            "oro_destroy": (None, [_vp]),
            "oro_max_depth": (_u32, [_vp]),
            "oro_node_count": (_u64, [_vp]),
            "oro_location_keys": (None, [_vp, _vp]),
            "oro_export_nodes": (None, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
            "oro_range": (_vp, [_vp, _vp, _u64, _int, _dbl]),
            "oro_pick": (_vp, [_vp, _vp, _u64, _dbl]),
            "oro_frustum": (_vp, [_vp, _vp, _u64, _u64, _dbl]),
            "oro_plane": (_vp, [_vp, _vp, _u64, _dbl, _int]),
            "oro_query": (_vp, [_vp, _vp, _vp, _u64, _vp, _vp, _vp, _int, _dbl]),
            "oro_knn": (_vp, [_vp, _vp, _u64, _vp, _dbl, _dbl]),
            "oro_ray": (_vp, [_vp, _vp, _u64, _dbl, _dbl, _dbl, _int]),
            "oro_collide_self": (_vp, [_vp, _dbl]),
            "oro_collide_pair": (_vp, [_vp, _vp, _dbl]),
            "oro_res_nq": (_u64, [_vp]),
            "oro_res_total": (_u64, [_vp]),
            "oro_res_has_dist": (_int, [_vp]),
            "oro_res_copy": (None, [_vp, _vp, _vp, _vp]),
            "oro_res_free": (None, [_vp]),
            "oro_time_create_points": (_dbl, [_vp, _u64, _u32, _u64, _int]),
            "oro_static": (_vp, [_vp]),
            "oro_static_sizes": (None, [_vp, _vp]),
            "oro_static_copy": (None, [_vp, _vp, _vp, _vp, _vp, _vp]),
            "oro_static_free": (None, [_vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        if hasattr(lib, "oro_brute_collide"):
            lib.oro_brute_collide.restype = _vp
            lib.oro_brute_collide.argtypes = [_int, _vp, _u64, _dbl]
        if hasattr(lib, "oro_create_threads"):
            lib.oro_create_threads.restype = _vp
            lib.oro_create_threads.argtypes = [_int, _int, _vp, _u64, _u32, _vp, _u64, _u32]
        if hasattr(lib, "oro_time_create_points_par"):
            lib.oro_time_create_points_par.restype = _dbl
            lib.oro_time_create_points_par.argtypes = [_vp, _u64, _u32, _u64, _int, _u32]
        if hasattr(lib, "oro_static_archive"):  # the reference harness only
            lib.oro_static_archive.restype = _u64
            lib.oro_static_archive.argtypes = [_vp, _int, _vp, _u64]
            lib.oro_static_load.restype = _vp
            lib.oro_static_load.argtypes = [_vp, _vp, _u64, _int]
            lib.oro_static_equal.restype = _int
            lib.oro_static_equal.argtypes = [_vp]
            lib.oro_dynamic_equals_static.restype = _int
            lib.oro_dynamic_equals_static.argtypes = [_vp]
        if hasattr(lib, "oro_node_parents"):
            lib.oro_node_parents.restype = None
            lib.oro_node_parents.argtypes = [_vp, _vp]
        if hasattr(lib, "oro_insert"):
            lib.oro_insert.restype = _int
            lib.oro_insert.argtypes = [_vp, _vp, _u64]
        if hasattr(lib, "oro_set_entities"):
            lib.oro_set_entities.restype = None
            lib.oro_set_entities.argtypes = [_vp, _vp, _u64]
        if hasattr(lib, "oro_count_work"):  # the restatement only
            lib.oro_count_work.restype = None
            lib.oro_count_work.argtypes = [_vp, _int]
            lib.oro_work.restype = None
            lib.oro_work.argtypes = [_vp, _vp]
        if hasattr(lib, "oro_collide_self_par"):
            lib.oro_collide_self_par.restype = _vp
            lib.oro_collide_self_par.argtypes = [_vp, _dbl]
        self.lib = lib

    # -------------------------------------------------------------- trees
    def create(self, ent, kind, max_depth=0, box=None, max_elem=16, threads=1):
        """threads > 1: the location transform and sort on that many workers (the oracle only)."""
        ent = np.ascontiguousarray(ent)
        scalar = 0 if ent.dtype == np.float64 else 1
        if box is not None:
            box = np.ascontiguousarray(box, dtype=ent.dtype)
        n = ent.shape[0] if ent.size else 0
        if threads > 1:
            h = self.lib.oro_create_threads(scalar, kind, _ptr(ent), n, max_depth, _ptr(box), max_elem, threads)
        else:
            h = self.lib.oro_create(scalar, kind, _ptr(ent), n, max_depth, _ptr(box), max_elem)
        return OracleTree(self, h, ent, kind)

    def brute_collide(self, boxes, tol=-1.0):
        boxes = np.ascontiguousarray(boxes)
        scalar = 0 if boxes.dtype == np.float64 else 1
        r = self.lib.oro_brute_collide(scalar, _ptr(boxes), boxes.shape[0], tol)
        off, ids, _ = self._result(r)
        return ids.reshape(-1, 2)

    def _result(self, r):
        nq = self.lib.oro_res_nq(r)
        tot = self.lib.oro_res_total(r)
        off = np.zeros(nq + 1, np.uint64)
        ids = np.zeros(tot, np.uint32)
        dist = np.zeros(tot, np.float64) if (self.lib.oro_res_has_dist(r) or tot == 0) else None
        self.lib.oro_res_copy(r, _ptr(off), _ptr(ids), _ptr(dist))
        self.lib.oro_res_free(r)
        return off, ids, dist


class OracleTree:
    def __init__(self, owner, handle, ent, kind):
        self.o = owner
        self.lib = owner.lib
        self.h = handle
        self.ent = ent
        self.kind = kind
        self.n = ent.shape[0] if ent.size else 0

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.oro_destroy(self.h)
            self.h = None

    @property
    def max_depth(self):
        return self.lib.oro_max_depth(self.h)

    @property
    def node_count(self):
        return self.lib.oro_node_count(self.h)

    def static_layout(self):
        """The static linear layout of the same entities (StaticLinearOrthoTreeCore's arrays), or
        None where it is undefined (a point tree holding points outside its space)."""
        h = self.lib.oro_static(self.h)
        if not h:
            return None
        try:
            sz = np.zeros(4, np.uint64)
            self.lib.oro_static_sizes(h, _ptr(sz))
            m, nb, ne, w = (int(v) for v in sz)
            cb = np.zeros(max(nb, 1), np.uint32)
            seg = np.zeros((max(m, 1), 2), np.uint32)
            dep = np.zeros(max(m, 1), np.uint8)
            es = np.zeros(max(ne, 1), np.uint32)
            geo = np.zeros((max(m, 1), w), np.float64)
            self.lib.oro_static_copy(h, _ptr(cb), _ptr(seg), _ptr(dep), _ptr(es), _ptr(geo))
        finally:
            self.lib.oro_static_free(h)
        return dict(child_begins=cb[:nb], segments=seg[:m], depth=dep[:m], entity_storage=es[:ne], geometry=geo[:m])

    def static_archive(self, managed=True):
        """The reference's own binary archive of its static tree of these entities (harness only)."""
        size = self.lib.oro_static_archive(self.h, int(managed), None, 0)
        buf = np.zeros(size, np.uint8)
        self.lib.oro_static_archive(self.h, int(managed), _ptr(buf), size)
        return buf.tobytes()

    def static_load(self, data, managed=True):
        """Loads archive bytes with the reference's BinaryInputArchive (harness only): None when
        they do not load, else (layout of the loaded tree, whether it IsEqualTo the reference's own
        tree of these entities and holds the same entities)."""
        buf = np.frombuffer(data, np.uint8).copy()
        h = self.lib.oro_static_load(self.h, _ptr(buf), buf.size, int(managed))
        if not h:
            return None
        equal = bool(self.lib.oro_static_equal(h))
        try:
            sz = np.zeros(4, np.uint64)
            self.lib.oro_static_sizes(h, _ptr(sz))
            m, nb, ne, w = (int(v) for v in sz)
            cb = np.zeros(max(nb, 1), np.uint32)
            seg = np.zeros((max(m, 1), 2), np.uint32)
            dep = np.zeros(max(m, 1), np.uint8)
            es = np.zeros(max(ne, 1), np.uint32)
            geo = np.zeros((max(m, 1), w), np.float64)
            self.lib.oro_static_copy(h, _ptr(cb), _ptr(seg), _ptr(dep), _ptr(es), _ptr(geo))
        finally:
            self.lib.oro_static_free(h)
        return dict(child_begins=cb[:nb], segments=seg[:m], depth=dep[:m], entity_storage=es[:ne], geometry=geo[:m]), equal

    def parents(self):
        """Parent key of every node (0 for the root), nodes in ascending key order (as nodes())."""
        out = np.zeros(self.node_count, np.uint64)
        self.lib.oro_node_parents(self.h, _ptr(out))
        return out

    def insert(self, ent):
        """Bulk Insert of new points (point trees); they get ids n .. n + len(ent) - 1. Returns the
        library's result (False: refused, nothing inserted)."""
        ent = np.ascontiguousarray(ent, dtype=self.ent.dtype)
        ok = bool(self.lib.oro_insert(self.h, _ptr(ent), ent.shape[0]))
        if ok:
            self.ent = np.concatenate([self.ent, ent])
            self.n = self.ent.shape[0]
        return ok

    def set_entities(self, ent):
        """Core form: the geometry later queries test (same count and layout; the tree keeps its nodes)."""
        ent = np.ascontiguousarray(ent, dtype=self.ent.dtype)
        assert ent.shape == self.ent.shape
        self.ent = ent
        self.lib.oro_set_entities(self.h, _ptr(ent), ent.shape[0] if ent.size else 0)
        return self

    def work(self, fn):
        """(node records, entity records, ids) that the reference's traversal reads and returns for
        the queries fn(self) runs (the restatement's counters; single-threaded)."""
        self.lib.oro_count_work(self.h, 1)
        try:
            fn(self)
            out = np.zeros(3, np.uint64)
            self.lib.oro_work(self.h, _ptr(out))
        finally:
            self.lib.oro_count_work(self.h, 0)
        return tuple(int(v) for v in out)

    def location_keys(self):
        out = np.zeros(self.n, np.uint64)
        self.lib.oro_location_keys(self.h, _ptr(out))
        return out

    def nodes(self):
        """Nodes sorted by key: keys, min (nn,3), size (nn,3), entity offsets, entity ids (ascending per node)."""
        nn = self.node_count
        keys = np.zeros(nn, np.uint64)
        minp = np.zeros((nn, 3), np.float64)
        size = np.zeros((nn, 3), np.float64)
        eoff = np.zeros(nn + 1, np.uint64)
        eids = np.zeros(max(self.n, 1), np.uint32)
        self.lib.oro_export_nodes(self.h, _ptr(keys), _ptr(minp), _ptr(size), _ptr(eoff), _ptr(eids), None)
        return dict(keys=keys, min=minp, size=size, eoff=eoff, eids=eids[: int(eoff[-1])])

    def _q(self, arr):
        return np.ascontiguousarray(arr, dtype=self.ent.dtype)

    def range_search(self, ranges, mode=0, tol=-1.0):
        ranges = self._q(ranges)
        return self.o._result(self.lib.oro_range(self.h, _ptr(ranges), ranges.shape[0], mode, tol))[:2]

    def pick_search(self, pts, tol=-1.0):
        pts = self._q(pts)
        return self.o._result(self.lib.oro_pick(self.h, _ptr(pts), pts.shape[0], tol))[:2]

    def frustum(self, planes, tol=-1.0):
        """planes: (nq, np, 4) as {origoDistance, nx, ny, nz}."""
        planes = self._q(planes)
        nq, np_ = planes.shape[0], planes.shape[1]
        return self.o._result(self.lib.oro_frustum(self.h, _ptr(planes), np_, nq, tol))[:2]

    def plane_search(self, planes, tol=-1.0):
        """planes: (nq, 4) as {origoDistance, nx, ny, nz}, one per query."""
        planes = self._q(planes)
        return self.o._result(self.lib.oro_plane(self.h, _ptr(planes), planes.shape[0], tol, 0))[:2]

    def plane_positive(self, planes, tol=-1.0):
        planes = self._q(planes)
        return self.o._result(self.lib.oro_plane(self.h, _ptr(planes), planes.shape[0], tol, 1))[:2]

    def query(self, conds, offsets, planes, crossing, boxes, or_op=False, tol=-1.0):
        """Combined queries: query q holds conds[offsets[q]:offsets[q+1]] (COND_DTYPE records);
        planes (n, 4), crossing (n,) uint8 per plane, boxes (m, 6)."""
        conds = np.ascontiguousarray(conds, COND_DTYPE)
        off = np.ascontiguousarray(offsets, np.uint64)
        planes = self._q(np.asarray(planes).reshape(-1, 4))
        cross = np.ascontiguousarray(crossing, np.uint8)
        boxes = self._q(np.asarray(boxes).reshape(-1, 6))
        return self.o._result(
            self.lib.oro_query(self.h, _ptr(conds), _ptr(off), len(off) - 1, _ptr(planes), _ptr(cross), _ptr(boxes), int(or_op), tol)
        )[:2]

    def knn(self, pts, k, max_dist=-1.0, tol=-1.0):
        pts = self._q(pts)
        kk = np.ascontiguousarray(np.broadcast_to(np.asarray(k, np.uint32), (pts.shape[0],)))
        return self.o._result(self.lib.oro_knn(self.h, _ptr(pts), pts.shape[0], _ptr(kk), max_dist, tol))

    def ray(self, rays, first=False, tol=-1.0, tol_inc=0.0, max_dist=-1.0):
        rays = self._q(rays)
        return self.o._result(self.lib.oro_ray(self.h, _ptr(rays), rays.shape[0], tol, tol_inc, max_dist, int(first)))

    def collide_self(self, tol=-1.0):
        return self.o._result(self.lib.oro_collide_self(self.h, tol))[1].reshape(-1, 2)

    def collide_self_par(self, tol=-1.0):
        return self.o._result(self.lib.oro_collide_self_par(self.h, tol))[1].reshape(-1, 2)

    def collide_pair(self, other, tol=-1.0):
        return self.o._result(self.lib.oro_collide_pair(self.h, other.h, tol))[1].reshape(-1, 2)


_cache = {}


def oracle():
    if "o" not in _cache:
        if not os.path.exists(ORACLE_SO):
            raise RuntimeError(f"oracle library missing: {ORACLE_SO} (run __graft_entry__.build())")
        _cache["o"] = OracleLib(ORACLE_SO)
    return _cache["o"]


def reference():
    """The reference itself (only where oracle/_ref was built from the reference sources)."""
    if "r" not in _cache:
        _cache["r"] = OracleLib(REF_SO) if os.path.exists(REF_SO) else None
    return _cache["r"]
