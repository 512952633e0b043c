/*
 * octree_gb300.h — C-ABI of the GB300 Morton location-code tree (OrthoTree's OctreePoint /
 * OctreeBox, Create + data-parallel queries) implemented with sm_103a CUDA kernels.
 *
 * The boundary takes plain pointers and sizes only. Every function returns an int status
 * (OTG_OK on success). Each entry point names the reference interface it replaces, with paths
 * relative to the OrthoTree project root.
 *
 * Memory spaces: inputs marked "mem" are host pointers (OTG_MEM_HOST; copied to the device
 * inside the call) or device pointers (OTG_MEM_DEVICE). Query results stay in device memory,
 * owned by an otg_result, until copied out with otg_result_copy().
 *
 * Scalars: a tree is OTG_SCALAR_F64 (double, the reference default BaseGeometryType) or
 * OTG_SCALAR_F32 (float); entity, query and plane arrays use the tree's scalar type.
 * Tolerance arguments are double; a negative tolerance selects the reference default
 * BASE_TOLERANCE = 100 * epsilon of the tree's scalar type (adapters/general.h:57).
 *
 * Layouts (all 3-D, arrays of structs exactly as the reference's types):
 *   point   : {x, y, z}                               PointND<3>       (adapters/general.h:346-347)
 *   box     : {min x, min y, min z, max x, max y, max z} BoundingBoxND<3> (adapters/general.h:349-354)
 *   ray     : {origin x, y, z, direction x, y, z}      RayND<3>         (adapters/general.h:356-361)
 *   plane   : {origo distance, normal x, y, z}         PlaneND<3>       (adapters/general.h:363-368)
 *
 * Streams: `stream` is a cudaStream_t (NULL = legacy default stream). Calls that return sizes to
 * the host synchronise that stream before returning.
 */
#ifndef OCTREE_GB300_H
#define OCTREE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OTG_OK 0
#define OTG_ERR_INVALID_ARGUMENT 1 /* misuse that the reference answers with ORTHOTREE_CRASH_IF / assert */
#define OTG_ERR_CUDA 2             /* a CUDA runtime call failed; see otg_last_error() */
#define OTG_ERR_OUT_OF_MEMORY 3
#define OTG_ERR_TIMEOUT 5          /* a bounded device-side wait ran out (never a hang) */
#define OTG_ERR_NOT_SUPPORTED 6
#define OTG_ERR_NO_DEVICE 7        /* no CUDA device: there is no CPU fallback */

#define OTG_MEM_HOST 0
#define OTG_MEM_DEVICE 1

#define OTG_SCALAR_F64 0
#define OTG_SCALAR_F32 1

/* tree kinds: core/ot_aliases.h:119 (OctreePoint) and :122 (OctreeBox) */
#define OTG_KIND_POINTS 0 /* loose factor 1.0, MinPoint node geometry (core/configuration.h:104-105) */
#define OTG_KIND_BOXES 1  /* loose factor 2.0, MBR node geometry      (core/configuration.h:107-108) */
#define OTG_KIND_BOXES_REGULAR 2 /* OrthoTreeBoxND<3, false> (core/ot_aliases.h:62-66): loose factor 1.0,
                                    MBR node geometry, box locations by GetBoxGridID (detail/si_grid.h:177-219) */

/* RangeSearchMode, core/types.h:83-87 */
#define OTG_RANGE_INSIDE 0
#define OTG_RANGE_OVERLAP 1

/* query-kernel variants: the plain one-query-per-thread FP64 kernels, and the batched kernels
   (warp per query, FP32 outward-rounded filter, FP64 recheck). Both return identical results. */
#define OTG_ALGO_DEFAULT 0
#define OTG_ALGO_PLAIN_FP64 1
#define OTG_ALGO_FILTERED 2

typedef struct otg_tree otg_tree;
typedef struct otg_result otg_result;

typedef struct otg_tree_info
{
  uint64_t entity_count;
  uint64_t node_count;
  uint32_t max_depth;   /* maxDepthID after EstimateMaxDepth (detail/utils.h:613-622) */
  uint32_t scalar;      /* OTG_SCALAR_* */
  uint32_t kind;        /* OTG_KIND_* */
  uint32_t n_trees;     /* trees of a forest (otg_forest_create), 0 for a single tree */
  uint64_t max_elements;
  double space_min[3];  /* the tree's space (given box or the entities' bounding box) */
  double space_max[3];
} otg_tree_info;

/* Last error message of the calling thread (empty when none). */
const char* otg_last_error(void);

/* Number of CUDA devices usable by the library (0: every compute call returns OTG_ERR_NO_DEVICE). */
int otg_device_count(void);

/* Allocates an empty tree object; replaces the default constructor of
   DynamicHashOrthoTreeCore (core/ot_dynamic_hash_core.h:333). */
int otg_tree_new(otg_tree** out, int scalar, int kind);
void otg_tree_free(otg_tree* tree);

/* (Re)builds the tree from n entities: the entity span of
   DynamicHashOrthoTreeCore::Create(entities, maxDepth, box, maxElementNo, exec)
   (core/ot_dynamic_hash_core.h:751-809) and the static Create(tree, ...) (:812-822), also reached
   through OrthoTreeManaged::Create (core/ot_managed.h:169-228, 318-360).
   max_depth 0 = estimate (EstimateMaxDepth); box NULL = the entities' bounding box.
   The entity array is copied into the tree (the Managed form's ownership, ot_managed.h:70-71);
   queries therefore need no entity argument. Asynchronous on `stream` unless mem == OTG_MEM_HOST,
   in which case the call returns after the build finished and reports device-side errors.
   With the environment variable OTG_L2_FETCH_BYTES set to a byte count, the first build of the
   process sets its CUDA context's L2 fetch granularity limit (cudaLimitMaxL2FetchGranularity) to it;
   unset or 0 leaves the limit unchanged. */
int otg_tree_create(otg_tree* tree, const void* entities, uint64_t n, uint32_t max_depth, const void* box, uint64_t max_elements, int mem,
                    void* stream);

/* Core (non-owning) form: the geometry that the tree's queries test from now on. The reference's
   Core trees take the entity span on every query (core/ot_query.h:424-427, 477-482, 1209-1215,
   1902-1906, with EntityContainerView = std::span<T const>, core/entity_adapter.h:171-174) and
   test the geometry of that span against the nodes that Create built from the earlier span. This
   call makes the GPU tree do the same: the nodes (and their boxes) stay as the last Create built
   them, and `entities` (n must equal the tree's entity count; the same layout as Create's) becomes
   the tested geometry. Host memory is copied; device memory is read once, here. Not for forests. */
int otg_tree_set_entities(otg_tree* tree, const void* entities, uint64_t n, int mem, void* stream);

/* Bulk Insert of points into a point tree, as DynamicHashOrthoTreeCore::Insert(newEntities,
   existingEntities) (core/ot_dynamic_hash_core.h:1012-1333; OrthoTreeManaged::Add(newEntities),
   core/ot_managed.h:421-455, calls it): the new points get the ids entity_count .. entity_count +
   n - 1 and join the tree without a rebuild. They are clustered by the reference's rule (sorted by
   location, split by 9 bits at a time, runs of at most 256 walked greedily, at most max_elements per
   new node where locations differ), each cluster joins the node at its location, created where
   missing, and new nodes are linked under their nearest ancestor with branch nodes where two of them
   claim one child slot (LinkOrphanNodes, :826-863). The tree keeps its space and max depth.
   entities: n * 3 scalars of the tree's type, host or device memory. Synchronises `stream`.
   OTG_ERR_INVALID_ARGUMENT (nothing inserted) when a point lies outside the tree's space, where the
   reference stores it with location code 0; OTG_ERR_NOT_SUPPORTED for box trees, forests and
   empty trees. A tree changed by Insert is refused by otg_tree_export_static. */
int otg_tree_insert(otg_tree* tree, const void* entities, uint64_t n, int mem, void* stream);

/* Waits for the tree's last build on `stream` and reports device-side errors (OTG_ERR_TIMEOUT). */
int otg_tree_sync(otg_tree* tree, void* stream);

int otg_tree_info_get(const otg_tree* tree, otg_tree_info* info);

/* Per-entity location keys (loc << 5 | depth, input order), as MortonGridSpaceIndexing::GetLocation
   and the compact Location storage produce them (detail/si_mortongrid.h:69-97, detail/si_morton.h:117-143).
   keys: device or host array of entity_count uint64. */
int otg_tree_export_locations(const otg_tree* tree, uint64_t* keys, int mem, void* stream);

/* The node set reachable from the root, in breadth-first order: node keys with sentinel bit
   (detail/si_morton.h:210-235), node min point and size as GetNodeMinPoint / GetNodeSize return them
   (core/ot_dynamic_hash_core.h:491-519), the node's own entity ids, child counts.
   keys[node_count], min_size[node_count*6] (double), entity_offsets[node_count+1],
   entity_ids[entity_count] (every reachable entity once), child_count[node_count]. Host memory. */
int otg_tree_export_nodes(const otg_tree* tree, uint64_t* keys, double* min_size, uint64_t* entity_offsets, uint32_t* entity_ids,
                          uint32_t* child_count);

/* The tree in the array layout of StaticLinearOrthoTreeCore (core/ot_static_linear_core.h:81-89),
   node for node as its parallel Create (:524-600) lays out the same entities: nodes breadth first,
   children in Morton order, each node below the root at the lowest common ancestor of its
   entities' locations, MinPoint (points) or MBR (boxes) node geometry. The arrays are those of
   GetNodes() (NodeStorageGeneral: 32-bit segment begins and lengths), GetNodeDepthIDs(),
   GetEntityStorage() and GetNodeGeometries(). entity_storage lists ids in location order; entities
   with equal locations are in id order, which the reference's unstable sort leaves unspecified. */
typedef struct otg_static_layout
{
  uint64_t node_count;
  uint64_t child_begin_count;      /* entries the reference stores: last node with children + 2; 1 without one; 0 when empty */
  uint64_t entity_count;
  uint32_t geometry_per_node;      /* scalars: 3 (points: min point) or 6 (boxes: min point, size) */
  uint32_t scalar_bytes;           /* 8 (double) or 4 (float): the tree's scalar type */
  const uint32_t* child_begins;    /* device: node_count + 1 entries; node i's children are [b[i], b[i+1]) */
  const uint32_t* entity_segments; /* device: {begin, length} per node, into entity_storage */
  const uint8_t* depth_ids;        /* device: node_count */
  const uint32_t* entity_storage;  /* device: entity_count */
  const void* geometry;            /* device: node_count * geometry_per_node scalars of the tree's type */
} otg_static_layout;

/* Computes the static layout of a single built tree on `stream` (synchronises it) and fills `out`
   with device pointers owned by the tree, valid until its next build, export or destruction.
   OTG_ERR_INVALID_ARGUMENT for a forest, and where the reference has no such tree: points outside
   the space of a point tree (its static Build does not end on them) or locations outside the grid. */
int otg_tree_export_static(otg_tree* tree, otg_static_layout* out, void* stream);

/* The tree as the reference's BinaryOutputArchive writes its static tree (`ar & tree`,
   serialization.h:359-385 with serialization/binary_archive.h and the headers of serialization/stl):
   StaticOctreePoint / StaticOctreeBox, or with with_entities != 0 the Managed
   StaticOctreePointM / StaticOctreeBoxM, which also holds the entities (serialization.h:433-438).
   The reference's BinaryInputArchive loads the bytes into that type. Little-endian scalars and
   32-bit size tags (serialized_size_t without ORTHOTREE__LARGE_DATASET, core/types.h:51-55); the
   node storage is the variant its Create picks. buffer NULL: only *size is set. A buffer shorter
   than the archive: OTG_ERR_INVALID_ARGUMENT with *size set. Host memory; synchronises `stream`.
   The same trees as otg_tree_export_static are refused. */
int otg_tree_save_static(otg_tree* tree, int with_entities, void* buffer, uint64_t capacity, uint64_t* size, void* stream);

/* Resumes a tree from a Managed archive (StaticOctreePointM / StaticOctreeBoxM, as written by the
   reference or by otg_tree_save_static with entities): its entities are rebuilt with the archived
   max depth and max elements per node, in `box` (NULL: the entities' bounding box, as Create
   without a box), and the rebuild is checked against every archived array (entity order within a
   node aside). OTG_ERR_INVALID_ARGUMENT for another tree type, a malformed archive, an archive
   without entities, or one whose tree is not the rebuild of its entities (the tree then holds
   that rebuild). `tree` gives the scalar type and kind (otg_tree_new); host memory. */
int otg_tree_load_static(otg_tree* tree, const void* buffer, uint64_t size, const void* box, void* stream);

/* Copies an exported static layout into host arrays (sizes as above; a null pointer skips an array). */
int otg_static_layout_copy(const otg_static_layout* layout, uint32_t* child_begins, uint32_t* entity_segments, uint8_t* depth_ids,
                           uint32_t* entity_storage, void* geometry);

/* ---------------------------------------------------------------- queries (batched) */

/* RangeSearch(range, entities, mode, tol) per query box (core/ot_query.h:476-583). */
int otg_range_search(const otg_tree* tree, const void* ranges, uint64_t n_queries, int mode, double tol, int algo, otg_result** out, int mem,
                     void* stream);

/* PickSearch(point, entities, tol) per query point (core/ot_query.h:425-466). */
int otg_pick_search(const otg_tree* tree, const void* points, uint64_t n_queries, double tol, int algo, otg_result** out, int mem, void* stream);

/* GetNearestNeighbors(point, k, maxDistanceWithin, entities, tol) (core/ot_query.h:1208-1270).
   k: n_queries uint32 (mem space of the points) or NULL with k_all for every query.
   max_distance < 0: unbounded (std::numeric_limits<Scalar>::max()). Results by (distance, id);
   more than k ids are returned when distances tie within the tolerance, as in the reference. */
int otg_knn(const otg_tree* tree, const void* points, uint64_t n_queries, const uint32_t* k, uint32_t k_all, double max_distance, double tol,
            int algo, otg_result** out, int mem, void* stream);

/* FrustumCulling(planes, entities, tol) (core/ot_query.h:767-833): planes_per_query planes per query. */
int otg_frustum_culling(const otg_tree* tree, const void* planes, uint64_t planes_per_query, uint64_t n_queries, double tol, int algo,
                        otg_result** out, int mem, void* stream);

/* PlaneSearch(distanceOfOrigo, planeNormal, entities, tol) (core/ot_query.h:612-636; the same as
   PlaneIntersection, :656-664): one plane {origoDistance, nx, ny, nz} (normalized) per query; the
   ids of the entities the plane hits, ascending per query. */
int otg_plane_search(const otg_tree* tree, const void* planes, uint64_t n_queries, double tol, int algo, otg_result** out, int mem, void* stream);

/* PlanePositiveSegmentation(distanceOfOrigo, planeNormal, entities, tol) (core/ot_query.h:687-744):
   one plane per query; the ids of the entities not on its negative side, ascending per query (a
   node wholly on the positive side contributes its subtree untested, as in the reference). */
int otg_plane_positive_segmentation(const otg_tree* tree, const void* planes, uint64_t n_queries, double tol, int algo, otg_result** out, int mem,
                                    void* stream);

/* One condition of a combined query, the QueryCondition variant of core/ot_query.h:835-861 without
   its callback alternatives (EntityIDCondition / EntityCondition cannot run on the GPU):
     OTG_COND_FRUSTUM       ByInFrustum: planes [first, first + count) of `planes`, each with its
                            isCrossingAllowed flag in `crossing_allowed`
     OTG_COND_RANGE_INSIDE  ByWithin: box `first` of `boxes`
     OTG_COND_RANGE_OVERLAP ByOverlaps: box `first` of `boxes`
     OTG_COND_PLANE         ByIntersecting: plane `first`, with its own tolerance `tol` (< 0: default) */
#define OTG_COND_FRUSTUM 0
#define OTG_COND_RANGE_INSIDE 1
#define OTG_COND_RANGE_OVERLAP 2
#define OTG_COND_PLANE 3
typedef struct otg_condition
{
  int32_t kind;
  uint32_t first;
  uint32_t count;
  uint32_t reserved; /* 0 */
  double tol;
} otg_condition;

/* Query<LogicalOperator::And / Or>(conditions, entities, tol) (core/ot_query.h:864-1026), batched:
   query q combines conditions[query_offsets[q] .. query_offsets[q + 1]) with AND (logical_or = 0)
   or OR (1). planes: n_planes planes, crossing_allowed: n_planes bytes, boxes: n_boxes boxes; all
   arrays, conditions and offsets included, in memory space `mem`. tol applies to the frustum and
   range conditions. Ids ascending per query. */
int otg_query(const otg_tree* tree, const otg_condition* conditions, const uint64_t* query_offsets, uint64_t n_queries, const void* planes,
              const uint8_t* crossing_allowed, uint64_t n_planes, const void* boxes, uint64_t n_boxes, int logical_or, double tol, int algo,
              otg_result** out, int mem, void* stream);

/* RayIntersectedAll(origin, direction, entities, tol, toleranceIncrement, maxExaminationDistance)
   (core/ot_query.h:1928-2022). max_distance < 0: unbounded; 0: no limit (reference semantics).
   Results by (enter distance, id). */
int otg_ray_all(const otg_tree* tree, const void* rays, uint64_t n_queries, double tol, double tol_increment, double max_distance, int algo,
                otg_result** out, int mem, void* stream);

/* RayIntersectedFirst(...) (core/ot_query.h:2035-2146). Results by (enter distance, id); the
   reference returns the same set farthest first. */
int otg_ray_first(const otg_tree* tree, const void* rays, uint64_t n_queries, double tol, double tol_increment, double max_distance, int algo,
                  otg_result** out, int mem, void* stream);

/* CollisionDetection(entities, tol, exec) within one box tree (core/ot_query.h:1690-1914).
   One result "query" whose ids are pairs (i, j), i < j, ascending. */
int otg_collision_self(const otg_tree* tree, double tol, int algo, otg_result** out, void* stream);

/* CollisionDetection(leftTree, leftEntities, rightTree, rightEntities, tol) (core/ot_query.h:1462-1497).
   Pairs (left id, right id), ascending. */
int otg_collision_pair(const otg_tree* left, const otg_tree* right, double tol, int algo, otg_result** out, void* stream);

/* kNN query that allocates no memory. No counterpart in the reference, whose
   GetNearestNeighbors (core/ot_query.h:1208-1270) answers one query with a freshly allocated
   std::vector. It exists for callers that cannot allocate device memory per call: frame loops
   with a fixed memory budget, code that must avoid the device-wide synchronisation that
   cudaMalloc/cudaFree imply, processes whose allocator is closed after start-up.
   The result equals otg_knn(..., k = NULL, k_all = k, ...): counts[q] is the number of ids the
   query has (ties within the tolerance can make it exceed k); the first min(counts[q],
   slot_capacity) of them, by (distance, id), are written to ids[q * slot_capacity ...] and
   distances[q * slot_capacity ...]. counts[q] > slot_capacity tells the caller the slot was too
   small. points, counts, ids and distances must be device memory; the tree must have been
   synchronised (otg_tree_sync or any earlier query). The call returns after its kernels finished.
   Scratch: a fixed array in the library's static device memory (8 MiB + 256 bytes per device)
   holds one threshold per query, so n_queries is at most 1048576 (larger values return
   OTG_ERR_INVALID_ARGUMENT); k is at most 256. The first call on each device looks up the
   array's device address (with that device current); make that first call, for instance with
   n_queries = 0, which only does this set-up, before any stream capture begins. All calls on a
   device share the one scratch array: calls that overlap on the GPU (from several host threads
   or streams) race on it, so the caller must serialise them. When the call returns an error,
   counts, ids and distances hold no defined values. */
int otg_knn_noalloc(const otg_tree* tree, const void* points, uint64_t n_queries, uint32_t k, double max_distance, double tol,
                    uint32_t slot_capacity, uint32_t* counts, uint32_t* ids, double* distances, void* stream);

/* ---------------------------------------------------------------- forests: many independent trees
   Builds n_trees independent trees in one launch sequence; no counterpart as one call in the
   reference, where each tree is its own Create (core/ot_dynamic_hash_core.h:751-822). Tree t is
   the Create of entities [tree_offsets[t], tree_offsets[t+1]) of `entities`, with max_depth
   (0: EstimateMaxDepth of that tree's size), its box boxes[t] (boxes NULL: its entities'
   bounding box) and max_elements. tree_offsets: n_trees + 1 host values starting at 0.
   Queries of forest t return the ids that tree t's own Create would give (0 .. size - 1). */
int otg_forest_create(otg_tree* tree, const void* entities, const uint64_t* tree_offsets, uint32_t n_trees, uint32_t max_depth, const void* boxes,
                      uint64_t max_elements, int mem, void* stream);
/* tree of every node (node_count uint32, host), e.g. to split otg_tree_export_nodes per tree */
int otg_forest_node_trees(const otg_tree* tree, uint32_t* node_tree);
/* The single-tree queries above, answered for many trees in one call: queries
   [query_offsets[t], query_offsets[t+1]) ask tree t (n_trees + 1 host values starting at 0);
   results are per query in that order. */
int otg_forest_range_search(const otg_tree* tree, const void* ranges, const uint64_t* query_offsets, int mode, double tol, int algo, otg_result** out,
                            int mem, void* stream);
int otg_forest_pick_search(const otg_tree* tree, const void* points, const uint64_t* query_offsets, double tol, int algo, otg_result** out, int mem,
                           void* stream);
int otg_forest_knn(const otg_tree* tree, const void* points, const uint64_t* query_offsets, const uint32_t* k, uint32_t k_all, double max_distance,
                   double tol, int algo, otg_result** out, int mem, void* stream);
int otg_forest_frustum_culling(const otg_tree* tree, const void* planes, uint64_t planes_per_query, const uint64_t* query_offsets, double tol, int algo,
                               otg_result** out, int mem, void* stream);
int otg_forest_ray_all(const otg_tree* tree, const void* rays, const uint64_t* query_offsets, double tol, double tol_increment, double max_distance,
                       int algo, otg_result** out, int mem, void* stream);
int otg_forest_ray_first(const otg_tree* tree, const void* rays, const uint64_t* query_offsets, double tol, double tol_increment, double max_distance,
                         int algo, otg_result** out, int mem, void* stream);

/* ---------------------------------------------------------------- recorded forest steps (CUDA graph)
   No counterpart in the reference. A plan records one step of a forest workload as a CUDA graph:
   the forest Create of `entities` (device memory, tree sizes given by tree_offsets) followed by
   the batched range search, ray-all (unbounded) and frustum queries of the given device inputs
   (any of the three may be NULL with its offsets NULL). otg_forest_plan_new runs the step once
   through the ordinary calls, sizes every result buffer at capacity_factor times that run's
   result count, and records the step. otg_forest_plan_run replays it on `stream`: the inputs are
   re-read from the same device buffers, so a caller updates them in place between runs.
   otg_forest_plan_result waits for the run and returns device pointers to the CSR result
   (which: 0 range, 1 ray-all, 2 frustum), valid until the next run; OTG_ERR_OUT_OF_MEMORY if the
   results outgrew the capacity. The plan uses `tree` until it is freed. */
typedef struct otg_plan otg_plan;
int otg_forest_plan_new(otg_plan** plan, otg_tree* tree, const void* entities, const uint64_t* tree_offsets, uint32_t n_trees, uint32_t max_depth,
                        uint64_t max_elements, const void* ranges, const uint64_t* range_offsets, int mode, const void* rays,
                        const uint64_t* ray_offsets, const void* planes, uint64_t planes_per_query, const uint64_t* frustum_offsets, double tol,
                        double capacity_factor, void* stream);
int otg_forest_plan_run(otg_plan* plan, void* stream);
int otg_forest_plan_result(otg_plan* plan, int which, uint64_t* n_queries, uint64_t* n_ids, const uint64_t** offsets, const uint32_t** ids,
                           const double** distances, void* stream);
/* copies the last run's result `which` into caller arrays (offsets[n_queries+1], ids[n_ids],
   distances[n_ids] or NULL; mem: destination space) */
int otg_forest_plan_copy(otg_plan* plan, int which, uint64_t* offsets, uint32_t* ids, double* distances, int mem, void* stream);
void otg_forest_plan_free(otg_plan* plan);

/* ---------------------------------------------------------------- results */
int otg_result_info(const otg_result* r, uint64_t* n_queries, uint64_t* n_ids, int* has_distances);
/* offsets[n_queries+1], ids[n_ids], distances[n_ids] (double; may be NULL). mem: destination space. */
int otg_result_copy(const otg_result* r, uint64_t* offsets, uint32_t* ids, double* distances, int mem, void* stream);
/* Device pointers owned by the result (valid until otg_result_free). The arrays come from the
   device's stream-ordered memory pool; otg_result_free returns them in the order of the legacy
   default stream, so work of the caller's that reads them on another stream must be complete, or
   ordered before that stream, when the result is freed. */
int otg_result_device_ptrs(const otg_result* r, const uint64_t** offsets, const uint32_t** ids, const double** distances);
/* Statistics of the last query that produced r: FP32-filter tests and FP64 rechecks. */
int otg_result_stats(const otg_result* r, uint64_t* filter_tests, uint64_t* fp64_rechecks);
void otg_result_free(otg_result* r);

/* ---------------------------------------------------------------- kernel-shape autotuning
   No counterpart in the reference. Query kernels exist in shapes that return identical results
   (one query per thread or per warp; 2, 4 or 8 warps per block; for the batched range, pick,
   frustum, plane, Query and ray kernels also the depth, none or 1-3, at which a batch's subtrees
   become separate work items). With autotuning on (the default) the first call of a query kind on
   a size class (kind, scalar, log2 entity count, log2 query count) times every shape on that
   call's own work and keeps the fastest for the class.
   otg_autotune_entry describes entry `index`: the class, each shape's time and the choice. */
int otg_autotune_enable(int on);
int otg_autotune_count(void);
int otg_autotune_entry(int index, char* text, int capacity);
/* Diagnostic: every tuned call whose candidate shapes include `shape` runs that shape (shape -1:
   back to tuning). Shapes of the batched query kernels: warps per block (2, 4, 8) | split << 8,
   split 1 = no split, 2-4 = subtrees at depth 1-3 become work items; 0 = one query per thread. */
int otg_autotune_force_shape(int shape);

/* ---------------------------------------------------------------- instrumentation
   No counterpart in the reference. When enabled, each otg_tree_create records a CUDA event on
   its stream before every build phase; after the stream has completed, otg_profile_phase()
   returns the phase names and their device durations (ms) of the last build. */
int otg_profile_enable(int on);
int otg_profile_phase_count(void);
int otg_profile_phase(int index, char* name, int name_capacity, float* milliseconds);

#ifdef __cplusplus
}
#endif

#endif /* OCTREE_GB300_H */
