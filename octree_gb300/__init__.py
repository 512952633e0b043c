"""Python host binding of the GB300 Morton location-code tree (C-ABI in include/octree_gb300.h).

The binding mirrors OrthoTree's Managed trees (OctreePointM / OctreeBoxM, core/ot_managed.h): the
tree owns a device copy of its entities, Create() rebuilds it, and every query is batched (one
call answers many query geometries). Inputs are numpy arrays (host) or torch CUDA tensors
(device). There is no CPU path: importing works anywhere, but every compute call raises
OtgError when the CUDA library or a GPU is missing.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboctree_gb300.so")

OTG_OK = 0
MEM_HOST, MEM_DEVICE = 0, 1
SCALAR_F64, SCALAR_F32 = 0, 1
KIND_POINTS, KIND_BOXES, KIND_BOXES_REGULAR = 0, 1, 2
RANGE_INSIDE, RANGE_OVERLAP = 0, 1
ALGO_DEFAULT, ALGO_PLAIN_FP64, ALGO_FILTERED = 0, 1, 2
# one condition of a combined query: the otg_condition record (include/octree_gb300.h)
COND_DTYPE = np.dtype([("kind", "<i4"), ("first", "<u4"), ("count", "<u4"), ("reserved", "<u4"), ("tol", "<f8")])
COND_FRUSTUM, COND_RANGE_INSIDE, COND_RANGE_OVERLAP, COND_PLANE = 0, 1, 2, 3

_STATUS = {
    1: "invalid argument",
    2: "CUDA error",
    3: "out of memory",
    5: "device wait timed out",
    6: "not supported",
    7: "no CUDA device",
}

_vp, _u64, _u32, _dbl, _int = C.c_void_p, C.c_uint64, C.c_uint32, C.c_double, C.c_int

# (name, restype, argtypes) of every exported entry point, in include/octree_gb300.h order
EXPORTS = [
    ("otg_last_error", C.c_char_p, []),
    ("otg_device_count", _int, []),
    ("otg_tree_new", _int, [C.POINTER(_vp), _int, _int]),
    ("otg_tree_free", None, [_vp]),
    ("otg_tree_create", _int, [_vp, _vp, _u64, _u32, _vp, _u64, _int, _vp]),
    ("otg_tree_set_entities", _int, [_vp, _vp, _u64, _int, _vp]),
    ("otg_tree_insert", _int, [_vp, _vp, _u64, _int, _vp]),
    ("otg_tree_sync", _int, [_vp, _vp]),
    ("otg_tree_info_get", _int, [_vp, _vp]),
    ("otg_tree_export_locations", _int, [_vp, _vp, _int, _vp]),
    ("otg_tree_export_nodes", _int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("otg_tree_export_static", _int, [_vp, _vp, _vp]),
    ("otg_tree_save_static", _int, [_vp, _int, _vp, _u64, C.POINTER(_u64), _vp]),
    ("otg_tree_load_static", _int, [_vp, _vp, _u64, _vp, _vp]),
    ("otg_static_layout_copy", _int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    ("otg_range_search", _int, [_vp, _vp, _u64, _int, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_pick_search", _int, [_vp, _vp, _u64, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_knn", _int, [_vp, _vp, _u64, _vp, _u32, _dbl, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_frustum_culling", _int, [_vp, _vp, _u64, _u64, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_plane_search", _int, [_vp, _vp, _u64, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_plane_positive_segmentation", _int, [_vp, _vp, _u64, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_query", _int, [_vp, _vp, _vp, _u64, _vp, _vp, _u64, _vp, _u64, _int, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_ray_all", _int, [_vp, _vp, _u64, _dbl, _dbl, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_ray_first", _int, [_vp, _vp, _u64, _dbl, _dbl, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_collision_self", _int, [_vp, _dbl, _int, C.POINTER(_vp), _vp]),
    ("otg_collision_pair", _int, [_vp, _vp, _dbl, _int, C.POINTER(_vp), _vp]),
    ("otg_knn_noalloc", _int, [_vp, _vp, _u64, _u32, _dbl, _dbl, _u32, _vp, _vp, _vp, _vp]),
    ("otg_forest_create", _int, [_vp, _vp, _vp, _u32, _u32, _vp, _u64, _int, _vp]),
    ("otg_forest_node_trees", _int, [_vp, _vp]),
    ("otg_forest_range_search", _int, [_vp, _vp, _vp, _int, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_forest_pick_search", _int, [_vp, _vp, _vp, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_forest_knn", _int, [_vp, _vp, _vp, _vp, _u32, _dbl, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_forest_frustum_culling", _int, [_vp, _vp, _u64, _vp, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_forest_ray_all", _int, [_vp, _vp, _vp, _dbl, _dbl, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_forest_ray_first", _int, [_vp, _vp, _vp, _dbl, _dbl, _dbl, _int, C.POINTER(_vp), _int, _vp]),
    ("otg_forest_plan_new", _int, [C.POINTER(_vp), _vp, _vp, _vp, _u32, _u32, _u64, _vp, _vp, _int, _vp, _vp, _vp, _u64, _vp, _dbl, _dbl, _vp]),
    ("otg_forest_plan_run", _int, [_vp, _vp]),
    ("otg_forest_plan_result", _int, [_vp, _int, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_vp), C.POINTER(_vp), C.POINTER(_vp), _vp]),
    ("otg_forest_plan_copy", _int, [_vp, _int, _vp, _vp, _vp, _int, _vp]),
    ("otg_forest_plan_free", None, [_vp]),
    ("otg_result_info", _int, [_vp, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_int)]),
    ("otg_result_copy", _int, [_vp, _vp, _vp, _vp, _int, _vp]),
    ("otg_result_device_ptrs", _int, [_vp, _vp, _vp, _vp]),
    ("otg_result_stats", _int, [_vp, C.POINTER(_u64), C.POINTER(_u64)]),
    ("otg_result_free", None, [_vp]),
    ("otg_autotune_enable", _int, [_int]),
    ("otg_autotune_count", _int, []),
    ("otg_autotune_entry", _int, [_int, C.c_char_p, _int]),
    ("otg_autotune_force_shape", _int, [_int]),
    ("otg_profile_enable", _int, [_int]),
    ("otg_profile_phase_count", _int, []),
    ("otg_profile_phase", _int, [_int, C.c_char_p, _int, C.POINTER(C.c_float)]),
]


class OtgError(RuntimeError):
    pass


class _TreeInfo(C.Structure):
    _fields_ = [
        ("entity_count", _u64),
        ("node_count", _u64),
        ("max_depth", _u32),
        ("scalar", _u32),
        ("kind", _u32),
        ("n_trees", _u32),
        ("max_elements", _u64),
        ("space_min", _dbl * 3),
        ("space_max", _dbl * 3),
    ]


class StaticLayout(C.Structure):
    """otg_static_layout: the device arrays of the static linear layout (include/octree_gb300.h)."""

    _fields_ = [
        ("node_count", _u64),
        ("child_begin_count", _u64),
        ("entity_count", _u64),
        ("geometry_per_node", _u32),
        ("scalar_bytes", _u32),
        ("child_begins", _vp),
        ("entity_segments", _vp),
        ("depth_ids", _vp),
        ("entity_storage", _vp),
        ("geometry", _vp),
    ]


_lib = None


def library():
    """Loads the CUDA library built by __graft_entry__.build(); raises when it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OtgError(f"CUDA library not built: {LIB_PATH} (run __graft_entry__.build())")
        lib = C.CDLL(LIB_PATH)
        for name, res, args in EXPORTS:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _check(rc):
    if rc != OTG_OK:
        msg = library().otg_last_error().decode(errors="replace")
        raise OtgError(f"{_STATUS.get(rc, rc)}: {msg}")


def device_count():
    return library().otg_device_count()


def autotune_enable(on=True):
    _check(library().otg_autotune_enable(1 if on else 0))


def autotune_force_shape(shape):
    """Runs `shape` in every tuned call that offers it (-1: back to tuning); shapes of the batched
    query kernels are warps per block (2, 4, 8) | split << 8 (1: no split, 2-4: split depth 1-3)."""
    _check(library().otg_autotune_force_shape(int(shape)))


def autotune_entries():
    """[text] of the autotuner's choices so far: size class, time of each shape, chosen shape."""
    lib = library()
    out = []
    for i in range(lib.otg_autotune_count()):
        buf = C.create_string_buffer(512)
        _check(lib.otg_autotune_entry(i, buf, 512))
        out.append(buf.value.decode())
    return out


def profile_enable(on=True):
    _check(library().otg_profile_enable(1 if on else 0))


def profile_phases():
    """[(phase name, device ms)] of the last build (after its stream completed)."""
    lib = library()
    out = []
    for i in range(lib.otg_profile_phase_count()):
        buf = C.create_string_buffer(64)
        ms = C.c_float()
        _check(lib.otg_profile_phase(i, buf, 64, C.byref(ms)))
        out.append((buf.value.decode(), ms.value))
    return out


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _arg(a, dtype):
    """(pointer, mem space, keepalive) of an array argument in the tree's scalar type."""
    if a is None:
        return None, MEM_HOST, None
    if _is_torch(a):
        import torch

        tdt = torch.float64 if dtype == np.float64 else (torch.float32 if dtype == np.float32 else torch.uint32)
        if a.dtype != tdt:
            a = a.to(tdt)
        a = a.contiguous()
        return C.c_void_p(a.data_ptr()), (MEM_DEVICE if a.is_cuda else MEM_HOST), a
    a = np.ascontiguousarray(a, dtype=dtype)
    return a.ctypes.data_as(_vp), MEM_HOST, a


def _stream_ptr(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class Result:
    """Owner of a device result (CSR offsets + ids [+ distances])."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None):
            library().otg_result_free(self.h)
            self.h = None

    def sizes(self):
        nq, nids, hd = _u64(), _u64(), _int()
        _check(library().otg_result_info(self.h, C.byref(nq), C.byref(nids), C.byref(hd)))
        return nq.value, nids.value, bool(hd.value)

    def stats(self):
        a, b = _u64(), _u64()
        _check(library().otg_result_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def to_host(self, stream=None):
        nq, nids, hd = self.sizes()
        off = np.zeros(nq + 1, np.uint64)
        ids = np.zeros(max(nids, 1), np.uint32)
        dist = np.zeros(max(nids, 1), np.float64) if hd else None
        _check(
            library().otg_result_copy(
                self.h, off.ctypes.data_as(_vp), ids.ctypes.data_as(_vp), None if dist is None else dist.ctypes.data_as(_vp), MEM_HOST, _stream_ptr(stream)
            )
        )
        return off, ids[:nids], (dist[:nids] if dist is not None else None)


class Tree:
    """A GPU OctreePoint (kind='points'), OctreeBox (kind='boxes', loose factor 2.0) or a regular
    box tree OrthoTreeBoxND<3, false> (kind='regular_boxes', loose factor 1.0)."""

    _KINDS = {"points": KIND_POINTS, "boxes": KIND_BOXES, "regular_boxes": KIND_BOXES_REGULAR}

    def __init__(self, kind="points", dtype=np.float64):
        if kind not in self._KINDS:
            raise ValueError(f"kind must be one of {sorted(self._KINDS)}")
        self.kind = self._KINDS[kind]
        self.dtype = np.dtype(dtype).type
        self.scalar = SCALAR_F64 if self.dtype == np.float64 else SCALAR_F32
        h = _vp()
        _check(library().otg_tree_new(C.byref(h), self.scalar, self.kind))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            library().otg_tree_free(self.h)
            self.h = None

    # ------------------------------------------------------------------ Create
    def create(self, entities, max_depth=0, box=None, max_elements=16, stream=None):
        """OrthoTree Create(entities, maxDepth, box, maxElementNo) — core/ot_dynamic_hash_core.h:751-822."""
        p, mem, keep = _arg(entities, self.dtype)
        n = int(entities.shape[0]) if len(entities.shape) else 0
        bp, bmem, bkeep = _arg(box, self.dtype)
        if box is not None and bmem != mem:
            bb = np.ascontiguousarray(box.cpu().numpy() if _is_torch(box) else box, dtype=self.dtype)
            if mem == MEM_DEVICE:
                import torch

                bkeep = torch.as_tensor(bb, device="cuda")
                bp = C.c_void_p(bkeep.data_ptr())
            else:
                bkeep = bb
                bp = bb.ctypes.data_as(_vp)
        _check(library().otg_tree_create(self.h, p, n, max_depth, bp, max_elements, mem, _stream_ptr(stream)))
        self._keep = (keep, bkeep)
        return self

    def set_entities(self, entities, stream=None):
        """Core form: the geometry that later queries test, as the reference's Core queries take the
        entity span on every call; the nodes stay as the last create() built them."""
        p, mem, keep = _arg(entities, self.dtype)
        n = int(entities.shape[0]) if len(entities.shape) else 0
        _check(library().otg_tree_set_entities(self.h, p, n, mem, _stream_ptr(stream)))
        self._keep_span = keep  # device input is read by the stream-ordered gather of this call
        return self

    def insert(self, entities, stream=None):
        """Bulk Insert of points (DynamicHashOrthoTreeCore::Insert, core/ot_dynamic_hash_core.h:1012):
        the new points get ids entity_count .. entity_count + len - 1. Raises (nothing inserted) when
        a point lies outside the tree's space."""
        p, mem, keep = _arg(entities, self.dtype)
        n = int(entities.shape[0]) if len(entities.shape) else 0
        _check(library().otg_tree_insert(self.h, p, n, mem, _stream_ptr(stream)))
        del keep  # the call synchronises its stream
        return self

    def sync(self, stream=None):
        _check(library().otg_tree_sync(self.h, _stream_ptr(stream)))

    def info(self):
        info = _TreeInfo()
        _check(library().otg_tree_info_get(self.h, C.byref(info)))
        return info

    @property
    def max_depth(self):
        return self.info().max_depth

    @property
    def node_count(self):
        return self.info().node_count

    def location_keys(self):
        n = self.info().entity_count
        out = np.zeros(max(n, 1), np.uint64)
        _check(library().otg_tree_export_locations(self.h, out.ctypes.data_as(_vp), MEM_HOST, None))
        return out[:n]

    def nodes(self):
        info = self.info()
        m, n = info.node_count, info.entity_count
        keys = np.zeros(m, np.uint64)
        ms = np.zeros((m, 6), np.float64)
        eoff = np.zeros(m + 1, np.uint64)
        eids = np.zeros(max(n, 1), np.uint32)
        cc = np.zeros(m, np.uint32)
        _check(
            library().otg_tree_export_nodes(
                self.h, keys.ctypes.data_as(_vp), ms.ctypes.data_as(_vp), eoff.ctypes.data_as(_vp), eids.ctypes.data_as(_vp), cc.ctypes.data_as(_vp)
            )
        )
        return dict(keys=keys, min=ms[:, :3], size=ms[:, 3:], eoff=eoff, eids=eids[: int(eoff[-1])], child_count=cc)

    def export_static(self, stream=None):
        """The tree in StaticLinearOrthoTreeCore's array layout (core/ot_static_linear_core.h),
        copied to the host: child_begins as the reference stores them, entity segments
        (begin, length), depth ids, entity storage and node geometry (MinPoint per node for points,
        MBR min and size for boxes), in the tree's scalar type."""
        lay = StaticLayout()
        _check(library().otg_tree_export_static(self.h, C.byref(lay), _stream_ptr(stream)))
        m, ne, w = lay.node_count, lay.entity_count, lay.geometry_per_node
        cb = np.zeros(m + 1, np.uint32)
        seg = np.zeros((m, 2), np.uint32)
        dep = np.zeros(m, np.uint8)
        es = np.zeros(ne, np.uint32)
        geo = np.zeros((m, w), self.dtype)
        ptr = lambda a: a.ctypes.data_as(_vp) if a.size else None
        _check(library().otg_static_layout_copy(C.byref(lay), ptr(cb), ptr(seg), ptr(dep), ptr(es), ptr(geo)))
        return dict(child_begins=cb[: lay.child_begin_count], child_begins_full=cb if m else cb[:0], segments=seg, depth=dep,
                    entity_storage=es, geometry=geo)

    def save_static(self, with_entities=True, stream=None):
        """The reference's binary archive of this tree's static form (bytes): StaticOctreePointM /
        StaticOctreeBoxM with the entities, or the core StaticOctreePoint / StaticOctreeBox."""
        size = _u64()
        _check(library().otg_tree_save_static(self.h, int(bool(with_entities)), None, 0, C.byref(size), _stream_ptr(stream)))
        buf = np.zeros(size.value, np.uint8)
        _check(library().otg_tree_save_static(self.h, int(bool(with_entities)), buf.ctypes.data_as(_vp), size.value, C.byref(size), _stream_ptr(stream)))
        return buf.tobytes()

    def load_static(self, archive, box=None, stream=None):
        """Resumes this tree from a Managed archive (see save_static): rebuilds the archived
        entities and checks the rebuild against the archive."""
        buf = np.frombuffer(archive, np.uint8)
        b = None if box is None else np.ascontiguousarray(box, dtype=self.dtype)
        _check(
            library().otg_tree_load_static(
                self.h, buf.ctypes.data_as(_vp) if buf.size else None, buf.size, None if b is None else b.ctypes.data_as(_vp), _stream_ptr(stream)
            )
        )
        return self

    # ------------------------------------------------------------------ queries
    def _query(self, name, args, mem, stream, raw):
        out = _vp()
        fn = getattr(library(), name)
        _check(fn(self.h, *args, C.byref(out), mem, _stream_ptr(stream)))
        r = Result(out)
        return r if raw else r.to_host(stream)

    def range_search(self, ranges, mode=RANGE_INSIDE, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(ranges, self.dtype)
        return self._query("otg_range_search", [p, int(ranges.shape[0]), mode, tol, algo], mem, stream, raw)

    def pick_search(self, points, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(points, self.dtype)
        return self._query("otg_pick_search", [p, int(points.shape[0]), tol, algo], mem, stream, raw)

    def knn(self, points, k, max_distance=-1.0, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(points, self.dtype)
        nq = int(points.shape[0])
        kp, kall, kkeep = None, 0, None
        if np.isscalar(k):
            kall = int(k)
        else:
            if _is_torch(k):
                import torch

                kkeep = k.to(torch.int32).contiguous()
                kp = C.c_void_p(kkeep.data_ptr())
            else:
                kkeep = np.ascontiguousarray(k, dtype=np.uint32)
                kp = kkeep.ctypes.data_as(_vp)
        return self._query("otg_knn", [p, nq, kp, kall, max_distance, tol, algo], mem, stream, raw)

    def frustum_culling(self, planes, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        """planes: (n_queries, planes_per_query, 4) as {origo distance, nx, ny, nz}."""
        p, mem, keep = _arg(planes, self.dtype)
        return self._query("otg_frustum_culling", [p, int(planes.shape[1]), int(planes.shape[0]), tol, algo], mem, stream, raw)

    def plane_search(self, planes, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        """PlaneSearch: planes (n_queries, 4) as {origo distance, nx, ny, nz}, one per query."""
        p, mem, keep = _arg(planes, self.dtype)
        return self._query("otg_plane_search", [p, int(planes.shape[0]), tol, algo], mem, stream, raw)

    def plane_positive_segmentation(self, planes, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        """PlanePositiveSegmentation: planes (n_queries, 4), one per query."""
        p, mem, keep = _arg(planes, self.dtype)
        return self._query("otg_plane_positive_segmentation", [p, int(planes.shape[0]), tol, algo], mem, stream, raw)

    def query(self, conds, offsets, planes=None, crossing=None, boxes=None, logical_or=False, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        """Query<And / Or>, batched: query q combines conds[offsets[q]:offsets[q+1]] (COND_DTYPE
        records); planes (n, 4) with crossing (n,) flags, boxes (m, 6). Host (numpy) inputs."""
        conds = np.ascontiguousarray(conds, COND_DTYPE)
        off = np.ascontiguousarray(offsets, np.uint64)
        pl = np.ascontiguousarray(np.zeros((0, 4)) if planes is None else planes, self.dtype).reshape(-1, 4)
        cr = np.ascontiguousarray(np.zeros(len(pl)) if crossing is None else crossing, np.uint8)
        bx = np.ascontiguousarray(np.zeros((0, 6)) if boxes is None else boxes, self.dtype).reshape(-1, 6)
        args = [conds.ctypes.data_as(_vp), off.ctypes.data_as(_vp), len(off) - 1, pl.ctypes.data_as(_vp), cr.ctypes.data_as(_vp), len(pl),
                bx.ctypes.data_as(_vp), len(bx), int(bool(logical_or)), tol, algo]
        return self._query("otg_query", args, MEM_HOST, stream, raw)

    def ray_all(self, rays, tol=-1.0, tol_increment=0.0, max_distance=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(rays, self.dtype)
        return self._query("otg_ray_all", [p, int(rays.shape[0]), tol, tol_increment, max_distance, algo], mem, stream, raw)

    def ray_first(self, rays, tol=-1.0, tol_increment=0.0, max_distance=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(rays, self.dtype)
        return self._query("otg_ray_first", [p, int(rays.shape[0]), tol, tol_increment, max_distance, algo], mem, stream, raw)

    def collision_self(self, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        out = _vp()
        _check(library().otg_collision_self(self.h, tol, algo, C.byref(out), _stream_ptr(stream)))
        r = Result(out)
        return r if raw else r.to_host(stream)[1].reshape(-1, 2)

    def collision_pair(self, other, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        out = _vp()
        _check(library().otg_collision_pair(self.h, other.h, tol, algo, C.byref(out), _stream_ptr(stream)))
        r = Result(out)
        return r if raw else r.to_host(stream)[1].reshape(-1, 2)


def _offsets(off):
    off = np.ascontiguousarray(off, dtype=np.uint64)
    return off.ctypes.data_as(_vp), off


class Forest(Tree):
    """Many independent trees built by one launch sequence (otg_forest_create): tree t holds the
    entities [tree_offsets[t], tree_offsets[t+1]) of one array. Queries name their tree through
    query_offsets (queries [query_offsets[t], query_offsets[t+1]) ask tree t) and return the ids
    tree t's own Create would give."""

    def create(self, entities, tree_offsets, max_depth=0, boxes=None, max_elements=16, stream=None):
        p, mem, keep = _arg(entities, self.dtype)
        op, okeep = _offsets(tree_offsets)
        bp, bmem, bkeep = _arg(boxes, self.dtype)
        if boxes is not None and bmem != mem:
            raise OtgError("entities and boxes must be in the same memory space")
        _check(library().otg_forest_create(self.h, p, op, len(okeep) - 1, max_depth, bp, max_elements, mem, _stream_ptr(stream)))
        self._keep = (keep, bkeep, okeep)
        return self

    @property
    def tree_count(self):
        return self.info().n_trees

    def node_trees(self):
        out = np.zeros(self.node_count, np.uint32)
        _check(library().otg_forest_node_trees(self.h, out.ctypes.data_as(_vp)))
        return out

    def _fquery(self, name, data, qoff, args, mem, stream, raw):
        op, okeep = _offsets(qoff)
        out = _vp()
        fn = getattr(library(), name)
        _check(fn(self.h, data, op, *args, C.byref(out), mem, _stream_ptr(stream)))
        r = Result(out)
        return r if raw else r.to_host(stream)

    def range_search(self, ranges, query_offsets, mode=RANGE_INSIDE, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(ranges, self.dtype)
        return self._fquery("otg_forest_range_search", p, query_offsets, [mode, tol, algo], mem, stream, raw)

    def pick_search(self, points, query_offsets, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(points, self.dtype)
        return self._fquery("otg_forest_pick_search", p, query_offsets, [tol, algo], mem, stream, raw)

    def knn(self, points, query_offsets, k, max_distance=-1.0, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(points, self.dtype)
        kp, kall, kkeep = None, 0, None
        if np.isscalar(k):
            kall = int(k)
        else:
            kkeep = np.ascontiguousarray(k, dtype=np.uint32) if not _is_torch(k) else k.to(__import__("torch").int32).contiguous()
            kp = kkeep.ctypes.data_as(_vp) if not _is_torch(k) else C.c_void_p(kkeep.data_ptr())
        return self._fquery("otg_forest_knn", p, query_offsets, [kp, kall, max_distance, tol, algo], mem, stream, raw)

    def frustum_culling(self, planes, query_offsets, tol=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        """planes: (n_queries, planes_per_query, 4) as {origo distance, nx, ny, nz}."""
        p, mem, keep = _arg(planes, self.dtype)
        op, okeep = _offsets(query_offsets)
        out = _vp()
        _check(library().otg_forest_frustum_culling(self.h, p, int(planes.shape[1]), op, tol, algo, C.byref(out), mem, _stream_ptr(stream)))
        r = Result(out)
        return r if raw else r.to_host(stream)

    def ray_all(self, rays, query_offsets, tol=-1.0, tol_increment=0.0, max_distance=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(rays, self.dtype)
        return self._fquery("otg_forest_ray_all", p, query_offsets, [tol, tol_increment, max_distance, algo], mem, stream, raw)

    def ray_first(self, rays, query_offsets, tol=-1.0, tol_increment=0.0, max_distance=-1.0, algo=ALGO_DEFAULT, stream=None, raw=False):
        p, mem, keep = _arg(rays, self.dtype)
        return self._fquery("otg_forest_ray_first", p, query_offsets, [tol, tol_increment, max_distance, algo], mem, stream, raw)


class ForestPlan:
    """One step of a forest workload recorded as a CUDA graph (otg_forest_plan_new): the forest
    Create of `entities` plus batched range search, ray-all and frustum queries, replayed by run().
    Inputs are torch CUDA tensors that run() re-reads; update them in place between runs."""

    RANGE, RAY_ALL, FRUSTUM = 0, 1, 2

    def __init__(self, forest, entities, tree_offsets, max_depth=0, max_elements=16, ranges=None, range_offsets=None, mode=RANGE_INSIDE,
                 rays=None, ray_offsets=None, planes=None, frustum_offsets=None, tol=-1.0, capacity_factor=1.5, stream=None):
        self.forest = forest
        self._keep = [entities, ranges, rays, planes]
        ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr())
        offs = []
        for o in (tree_offsets, range_offsets, ray_offsets, frustum_offsets):
            offs.append((None, None) if o is None else _offsets(o))
        self._offs = offs
        self._nq = [None if o is None else len(o) - 1 for o in (range_offsets, ray_offsets, frustum_offsets)]
        h = _vp()
        _check(library().otg_forest_plan_new(
            C.byref(h), forest.h, ptr(entities), offs[0][0], len(offs[0][1]) - 1, max_depth, max_elements, ptr(ranges), offs[1][0], mode,
            ptr(rays), offs[2][0], ptr(planes), 0 if planes is None else int(planes.shape[1]), offs[3][0], tol, capacity_factor, _stream_ptr(stream)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            library().otg_forest_plan_free(self.h)
            self.h = None

    def run(self, stream=None):
        _check(library().otg_forest_plan_run(self.h, _stream_ptr(stream)))

    def result(self, which, stream=None):
        """(offsets, ids, distances or None) of the last run, on the host."""
        nq, n = _u64(), _u64()
        o, i, d = _vp(), _vp(), _vp()
        _check(library().otg_forest_plan_result(self.h, which, C.byref(nq), C.byref(n), C.byref(o), C.byref(i), C.byref(d), _stream_ptr(stream)))
        off = np.zeros(nq.value + 1, np.uint64)
        ids = np.zeros(max(n.value, 1), np.uint32)
        dist = np.zeros(max(n.value, 1), np.float64) if which == self.RAY_ALL else None
        _check(library().otg_forest_plan_copy(self.h, which, off.ctypes.data_as(_vp), ids.ctypes.data_as(_vp),
                                              None if dist is None else dist.ctypes.data_as(_vp), MEM_HOST, _stream_ptr(stream)))
        return off, ids[: n.value], (dist[: n.value] if dist is not None else None)
