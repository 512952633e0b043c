// otg_capi.cu — the extern "C" boundary (include/octree_gb300.h).
//
// Every entry point validates its arguments, runs on the caller's stream and returns a status.
// There is no CPU path: without a CUDA device every compute call returns OTG_ERR_NO_DEVICE.
#include "otg_internal.h"

#include <algorithm>
#include <mutex>

#include <cstring>
#include <new>
#include <string>


namespace otg
{
static thread_local std::string g_lastError;

void set_error(const std::string& msg) { g_lastError = msg; }

void keep_pool_memory(int device)
{
  static std::mutex lock;
  static bool done[64] = {};
  if (device < 0 || device >= 64)
    return;
  std::lock_guard<std::mutex> g(lock);
  if (done[device])
    return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess)
  {
    // freed blocks up to 8 GiB stay in the pool (a 16M-point tree's arrays after an Insert take
    // about 1.1 GB), at most a sixteenth of the device's memory
    size_t freeB = 0, totalB = 0;
    cudaMemGetInfo(&freeB, &totalB);
    unsigned long long threshold = std::min<unsigned long long>(8ull << 30, totalB / 16);
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
  }
  cudaGetLastError();
  done[device] = true;
}

int cuda_status(cudaError_t e, const char* what)
{
  if (e == cudaSuccess)
    return OTG_OK;
  set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
  cudaGetLastError(); // clear the sticky-free error state
  return e == cudaErrorMemoryAllocation ? OTG_ERR_OUT_OF_MEMORY : OTG_ERR_CUDA;
}

Profiler& profiler()
{
  static Profiler p;
  return p;
}
void Profiler::reset()
{
  for (cudaEvent_t e : events)
    cudaEventDestroy(e);
  events.clear();
  names.clear();
}
void Profiler::mark(const char* name, cudaStream_t st)
{
  if (!enabled)
    return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess)
    return;
  cudaEventRecord(e, st);
  events.push_back(e);
  names.push_back(name);
}

static int require_device()
{
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
  {
    cudaGetLastError();
    set_error("no CUDA device is available; this library has no CPU path");
    return OTG_ERR_NO_DEVICE;
  }
  return OTG_OK;
}

static int require_tree(const otg_tree* t, bool built = true)
{
  if (!t)
  {
    set_error("tree is NULL");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (built && !t->s.built)
  {
    set_error("tree was not created");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  return OTG_OK;
}

// queries need the node count on the host (first query after an asynchronous build)
static int ready(const otg_tree* t, cudaStream_t st)
{
  if (int rc = require_tree(t))
    return rc;
  if (!t->s.countsKnown)
    return finish_build(const_cast<otg_tree*>(t)->s, st);
  return OTG_OK;
}

static int new_result(otg_result** out)
{
  if (!out)
  {
    set_error("result pointer is NULL");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  *out = new (std::nothrow) otg_result();
  if (!*out)
  {
    set_error("out of host memory");
    return OTG_ERR_OUT_OF_MEMORY;
  }
  return OTG_OK;
}

static void release_tree(TreeState& s)
{
  DevBuf* bufs[] = { &s.entities, &s.sortedIds, &s.sortedGeom, &s.keysA, &s.keysB, &s.valsB, &s.nodeLink, &s.nodeKey, &s.nodeBox,
                     &s.nodeMax, &s.nodeDepth, &s.levelCount, &s.space, &s.sortScratch, &s.err, &s.bboxBits, &s.locations, &s.boxDev, &s.ownerNode, &s.nodeParent, &s.rasterTab, &s.minTab, &s.splitQueue, &s.geom32, &s.nodeBox32, &s.treeOff, &s.treeD, &s.nodeTree, &s.tabOff, &s.minOff, &s.segTiles,
                     &s.stOrder, &s.stChildBegin, &s.stSeg, &s.stDepth, &s.stGeom, &s.stCtl };
  for (DevBuf* b : bufs)
    b->release();
  s.retired.clear();
}

// forest: the query addresses the trees of a forest (per-query trees) rather than a single tree
template<typename F>
static int run_query(const otg_tree* t, otg_result** out, cudaStream_t st, F&& f, bool forest = false)
{
  if (int rc = require_device())
    return rc;
  if (int rc = ready(t, st))
    return rc;
  if ((t->s.trees != 0) != forest)
  {
    set_error(forest ? "otg_forest_* queries need a tree built by otg_forest_create" : "a forest is queried with the otg_forest_* calls");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (int rc = new_result(out))
    return rc;
  int rc = f((*out)->s);
  if (rc)
  {
    delete *out;
    *out = nullptr;
  }
  return rc;
}
} // namespace otg

using namespace otg;

// forest queries: queries [query_offsets[t], query_offsets[t+1]) ask tree t (host offsets)
template<typename F>
static int forest_query(const otg_tree* t, const uint64_t* qoff, otg_result** out, void* stream, F&& f)
{
  return run_query(
    t, out, (cudaStream_t)stream,
    [&](ResultState& r) {
      DevBuf qoffDev, qTree;
      u64 nq = 0;
      if (int rc = forest_query_trees(t->s, qoff, qoffDev, qTree, nq, (cudaStream_t)stream))
        return rc;
      return f(r, nq, qTree.as<u32>());
    },
    true);
}


extern "C"
{
  const char* otg_last_error(void) { return g_lastError.c_str(); }

  int otg_device_count(void)
  {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess)
    {
      cudaGetLastError();
      return 0;
    }
    return n;
  }

  int otg_tree_new(otg_tree** out, int scalar, int kind)
  {
    if (!out || (scalar != OTG_SCALAR_F64 && scalar != OTG_SCALAR_F32) || (kind != OTG_KIND_POINTS && kind != OTG_KIND_BOXES && kind != OTG_KIND_BOXES_REGULAR))
    {
      set_error("otg_tree_new: invalid argument");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    *out = new (std::nothrow) otg_tree();
    if (!*out)
      return OTG_ERR_OUT_OF_MEMORY;
    (*out)->s.scalar = scalar;
    (*out)->s.kind = kind;
    return OTG_OK;
  }

  void otg_tree_free(otg_tree* t)
  {
    if (!t)
      return;
    release_tree(t->s);
    delete t;
  }

  int otg_tree_create(otg_tree* t, const void* entities, uint64_t n, uint32_t max_depth, const void* box, uint64_t max_elements, int mem, void* stream)
  {
    if (int rc = require_tree(t, false))
      return rc;
    if ((n && !entities) || (mem != OTG_MEM_HOST && mem != OTG_MEM_DEVICE))
    {
      set_error("otg_tree_create: invalid argument");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    if (int rc = require_device())
      return rc;
    return build_tree(t->s, entities, n, max_depth, box, max_elements, mem, (cudaStream_t)stream);
  }

  int otg_tree_set_entities(otg_tree* t, const void* entities, uint64_t n, int mem, void* stream)
  {
    if (int rc = ready(t, (cudaStream_t)stream))
      return rc;
    if ((n && !entities) || (mem != OTG_MEM_HOST && mem != OTG_MEM_DEVICE))
    {
      set_error("otg_tree_set_entities: invalid argument");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    if (int rc = require_device())
      return rc;
    return set_entities(t->s, entities, n, mem, (cudaStream_t)stream);
  }

  int otg_tree_insert(otg_tree* t, const void* entities, uint64_t n, int mem, void* stream)
  {
    if (int rc = ready(t, (cudaStream_t)stream))
      return rc;
    if ((n && !entities) || (mem != OTG_MEM_HOST && mem != OTG_MEM_DEVICE))
    {
      set_error("otg_tree_insert: invalid argument");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    if (int rc = require_device())
      return rc;
    return insert_points(t->s, entities, n, mem, (cudaStream_t)stream);
  }

  int otg_tree_sync(otg_tree* t, void* stream)
  {
    if (int rc = require_tree(t))
      return rc;
    return finish_build(t->s, (cudaStream_t)stream);
  }

  int otg_tree_info_get(const otg_tree* t, otg_tree_info* info)
  {
    if (int rc = require_tree(t))
      return rc;
    if (!info)
      return OTG_ERR_INVALID_ARGUMENT;
    if (int rc = ready(t, nullptr))
      return rc;
    std::memset(info, 0, sizeof(*info));
    info->entity_count = t->s.n;
    info->node_count = t->s.nodeCount;
    info->max_depth = t->s.D;
    info->scalar = uint32_t(t->s.scalar);
    info->kind = uint32_t(t->s.kind);
    info->n_trees = t->s.trees;
    info->max_elements = t->s.maxElem;
    if (t->s.n)
    {
      if (t->s.scalar == OTG_SCALAR_F64)
      {
        Space<double> sp;
        if (cudaMemcpy(&sp, t->s.space.p, sizeof(sp), cudaMemcpyDeviceToHost) == cudaSuccess)
          for (int c = 0; c < 3; ++c)
          {
            info->space_min[c] = sp.min[c];
            info->space_max[c] = sp.max[c];
          }
      }
      else
      {
        Space<float> sp;
        if (cudaMemcpy(&sp, t->s.space.p, sizeof(sp), cudaMemcpyDeviceToHost) == cudaSuccess)
          for (int c = 0; c < 3; ++c)
          {
            info->space_min[c] = sp.min[c];
            info->space_max[c] = sp.max[c];
          }
      }
    }
    return OTG_OK;
  }

  int otg_tree_export_locations(const otg_tree* t, uint64_t* keys, int mem, void* stream)
  {
    if (int rc = ready(t, (cudaStream_t)stream))
      return rc;
    if (!keys && t->s.n)
      return OTG_ERR_INVALID_ARGUMENT;
    return export_locations(t->s, keys, mem, (cudaStream_t)stream);
  }

  int otg_tree_export_nodes(const otg_tree* t, uint64_t* keys, double* min_size, uint64_t* entity_offsets, uint32_t* entity_ids, uint32_t* child_count)
  {
    if (int rc = ready(t, nullptr))
      return rc;
    if (!keys || !min_size || !entity_offsets || (!entity_ids && t->s.n))
      return OTG_ERR_INVALID_ARGUMENT;
    return export_nodes(t->s, keys, min_size, entity_offsets, entity_ids, child_count);
  }

  int otg_tree_export_static(otg_tree* t, otg_static_layout* out, void* stream)
  {
    if (int rc = require_device())
      return rc;
    if (int rc = ready(t, (cudaStream_t)stream))
      return rc;
    return export_static(t->s, out, (cudaStream_t)stream);
  }

  int otg_tree_save_static(otg_tree* t, int with_entities, void* buffer, uint64_t capacity, uint64_t* size, void* stream)
  {
    if (int rc = require_device())
      return rc;
    if (int rc = ready(t, (cudaStream_t)stream))
      return rc;
    if (!size)
    {
      set_error("otg_tree_save_static: null size");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    return save_static_archive(t->s, with_entities != 0, buffer, capacity, size, (cudaStream_t)stream);
  }

  int otg_tree_load_static(otg_tree* t, const void* buffer, uint64_t size, const void* box, void* stream)
  {
    if (int rc = require_tree(t, false))
      return rc;
    if (!buffer && size)
    {
      set_error("otg_tree_load_static: null buffer");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    if (int rc = require_device())
      return rc;
    return load_static_archive(t->s, buffer, size, box, (cudaStream_t)stream);
  }

  int otg_static_layout_copy(const otg_static_layout* l, uint32_t* child_begins, uint32_t* entity_segments, uint8_t* depth_ids, uint32_t* entity_storage,
                             void* geometry)
  {
    if (!l)
    {
      set_error("otg_static_layout_copy: null layout");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    const uint64_t m = l->node_count;
    const size_t scalar = l->scalar_bytes;
    struct Part
    {
      void* dst;
      const void* src;
      size_t bytes;
    } parts[] = { { child_begins, l->child_begins, m ? sizeof(uint32_t) * (m + 1) : 0 },
                  { entity_segments, l->entity_segments, sizeof(uint32_t) * 2 * m },
                  { depth_ids, l->depth_ids, m },
                  { entity_storage, l->entity_storage, sizeof(uint32_t) * l->entity_count },
                  { geometry, l->geometry, scalar * l->geometry_per_node * m } };
    for (const Part& p : parts)
      if (p.dst && p.bytes)
      {
        if (!p.src)
        {
          set_error("otg_static_layout_copy: the layout holds no such array");
          return OTG_ERR_INVALID_ARGUMENT;
        }
        if (cudaError_t e = cudaMemcpy(p.dst, p.src, p.bytes, cudaMemcpyDeviceToHost))
          return cuda_status(e, "copying the static layout");
      }
    return OTG_OK;
  }

  int otg_range_search(const otg_tree* t, const void* ranges, uint64_t nq, int mode, double tol, int algo, otg_result** out, int mem, void* stream)
  {
    if ((nq && !ranges) || (mode != OTG_RANGE_INSIDE && mode != OTG_RANGE_OVERLAP))
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream,
                     [&](ResultState& r) { return query_range(t->s, ranges, nq, mode, tol, algo, r, mem, (cudaStream_t)stream); });
  }

  int otg_pick_search(const otg_tree* t, const void* points, uint64_t nq, double tol, int algo, otg_result** out, int mem, void* stream)
  {
    if (nq && !points)
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream, [&](ResultState& r) { return query_pick(t->s, points, nq, tol, algo, r, mem, (cudaStream_t)stream); });
  }

  int otg_knn(const otg_tree* t, const void* points, uint64_t nq, const uint32_t* k, uint32_t k_all, double max_distance, double tol, int algo,
              otg_result** out, int mem, void* stream)
  {
    if (nq && !points)
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream,
                     [&](ResultState& r) { return query_knn(t->s, points, nq, k, k_all, max_distance, tol, algo, r, mem, (cudaStream_t)stream); });
  }

  int otg_frustum_culling(const otg_tree* t, const void* planes, uint64_t planes_per_query, uint64_t nq, double tol, int algo, otg_result** out, int mem,
                          void* stream)
  {
    if (nq && planes_per_query && !planes)
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream,
                     [&](ResultState& r) { return query_frustum(t->s, planes, planes_per_query, nq, tol, algo, r, mem, (cudaStream_t)stream); });
  }

  int otg_plane_search(const otg_tree* t, const void* planes, uint64_t nq, double tol, int algo, otg_result** out, int mem, void* stream)
  {
    if (nq && !planes)
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream, [&](ResultState& r) { return query_plane(t->s, planes, nq, false, tol, algo, r, mem, (cudaStream_t)stream); });
  }

  int otg_plane_positive_segmentation(const otg_tree* t, const void* planes, uint64_t nq, double tol, int algo, otg_result** out, int mem, void* stream)
  {
    if (nq && !planes)
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream, [&](ResultState& r) { return query_plane(t->s, planes, nq, true, tol, algo, r, mem, (cudaStream_t)stream); });
  }

  int otg_query(const otg_tree* t, const otg_condition* conditions, const uint64_t* query_offsets, uint64_t nq, const void* planes,
                const uint8_t* crossing_allowed, uint64_t n_planes, const void* boxes, uint64_t n_boxes, int logical_or, double tol, int algo,
                otg_result** out, int mem, void* stream)
  {
    static_assert(sizeof(otg_condition) == 24, "otg_condition is the 24-byte record the kernels read");
    if (nq && !query_offsets)
      return OTG_ERR_INVALID_ARGUMENT;
    if ((n_planes && (!planes || !crossing_allowed)) || (n_boxes && !boxes))
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream, [&](ResultState& r) {
      return query_combined(t->s, conditions, query_offsets, nq, planes, crossing_allowed, n_planes, boxes, n_boxes, logical_or, tol, algo, r, mem,
                            (cudaStream_t)stream);
    });
  }

  int otg_ray_all(const otg_tree* t, const void* rays, uint64_t nq, double tol, double tol_increment, double max_distance, int algo, otg_result** out,
                  int mem, void* stream)
  {
    if (nq && !rays)
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream, [&](ResultState& r) {
      return query_ray(t->s, rays, nq, tol, tol_increment, max_distance, false, algo, r, mem, (cudaStream_t)stream);
    });
  }

  int otg_ray_first(const otg_tree* t, const void* rays, uint64_t nq, double tol, double tol_increment, double max_distance, int algo, otg_result** out,
                    int mem, void* stream)
  {
    if (nq && !rays)
      return OTG_ERR_INVALID_ARGUMENT;
    return run_query(t, out, (cudaStream_t)stream, [&](ResultState& r) {
      return query_ray(t->s, rays, nq, tol, tol_increment, max_distance, true, algo, r, mem, (cudaStream_t)stream);
    });
  }

  int otg_collision_self(const otg_tree* t, double tol, int algo, otg_result** out, void* stream)
  {
    if (t && t->s.kind == OTG_KIND_POINTS)
    {
      set_error("collision detection needs a box tree");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    return run_query(t, out, (cudaStream_t)stream, [&](ResultState& r) { return query_collide_self(t->s, tol, algo, r, (cudaStream_t)stream); });
  }

  int otg_collision_pair(const otg_tree* a, const otg_tree* b, double tol, int algo, otg_result** out, void* stream)
  {
    if (int rc = ready(b, (cudaStream_t)stream))
      return rc;
    if (b->s.trees)
    {
      set_error("collision detection is defined for single trees, not forests");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    if ((a && a->s.kind == OTG_KIND_POINTS) || b->s.kind == OTG_KIND_POINTS || (a && a->s.kind != b->s.kind) || (a && a->s.scalar != b->s.scalar))
    {
      set_error("collision detection needs two box trees of the same scalar type");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    return run_query(a, out, (cudaStream_t)stream, [&](ResultState& r) { return query_collide_pair(a->s, b->s, tol, algo, r, (cudaStream_t)stream); });
  }

  int otg_knn_noalloc(const otg_tree* t, const void* points, uint64_t nq, uint32_t k, double max_distance, double tol, uint32_t slot_capacity,
                      uint32_t* counts, uint32_t* ids, double* distances, void* stream)
  {
    if (int rc = require_device())
      return rc;
    if (int rc = require_tree(t))
      return rc;
    if (!t->s.countsKnown)
    {
      set_error("the tree's build has not been synchronised (call otg_tree_sync first)");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    if (t->s.trees)
    {
      set_error("otg_knn_noalloc answers queries on a single tree, not a forest");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    return query_knn_noalloc(t->s, points, nq, k, max_distance, tol, slot_capacity, counts, ids, distances, (cudaStream_t)stream);
  }

  int otg_forest_create(otg_tree* t, const void* entities, const uint64_t* tree_offsets, uint32_t n_trees, uint32_t max_depth, const void* boxes,
                        uint64_t max_elements, int mem, void* stream)
  {
    if (int rc = require_tree(t, false))
      return rc;
    if ((!entities && tree_offsets && n_trees && tree_offsets[n_trees]) || (mem != OTG_MEM_HOST && mem != OTG_MEM_DEVICE))
    {
      set_error("otg_forest_create: invalid argument");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    if (int rc = require_device())
      return rc;
    return build_forest(t->s, entities, tree_offsets, n_trees, max_depth, boxes, max_elements, mem, (cudaStream_t)stream);
  }

  int otg_forest_node_trees(const otg_tree* t, uint32_t* node_tree)
  {
    if (int rc = ready(t, nullptr))
      return rc;
    if (!t->s.trees || !node_tree)
    {
      set_error("otg_forest_node_trees needs a forest and an output array");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    return cuda_status(cudaMemcpy(node_tree, t->s.nodeTree.p, sizeof(uint32_t) * t->s.nodeCount, cudaMemcpyDeviceToHost), "exporting node trees");
  }

  int otg_forest_range_search(const otg_tree* t, const void* ranges, const uint64_t* query_offsets, int mode, double tol, int algo, otg_result** out, int mem,
                              void* stream)
  {
    if (mode != OTG_RANGE_INSIDE && mode != OTG_RANGE_OVERLAP)
      return OTG_ERR_INVALID_ARGUMENT;
    return forest_query(t, query_offsets, out, stream, [&](ResultState& r, u64 nq, const u32* qt) {
      return query_range(t->s, ranges, nq, mode, tol, algo, r, mem, (cudaStream_t)stream, qt);
    });
  }

  int otg_forest_pick_search(const otg_tree* t, const void* points, const uint64_t* query_offsets, double tol, int algo, otg_result** out, int mem,
                             void* stream)
  {
    return forest_query(t, query_offsets, out, stream,
                        [&](ResultState& r, u64 nq, const u32* qt) { return query_pick(t->s, points, nq, tol, algo, r, mem, (cudaStream_t)stream, qt); });
  }

  int otg_forest_knn(const otg_tree* t, const void* points, const uint64_t* query_offsets, const uint32_t* k, uint32_t k_all, double max_distance,
                     double tol, int algo, otg_result** out, int mem, void* stream)
  {
    return forest_query(t, query_offsets, out, stream, [&](ResultState& r, u64 nq, const u32* qt) {
      return query_knn(t->s, points, nq, k, k_all, max_distance, tol, algo, r, mem, (cudaStream_t)stream, qt);
    });
  }

  int otg_forest_frustum_culling(const otg_tree* t, const void* planes, uint64_t planes_per_query, const uint64_t* query_offsets, double tol, int algo,
                                 otg_result** out, int mem, void* stream)
  {
    return forest_query(t, query_offsets, out, stream, [&](ResultState& r, u64 nq, const u32* qt) {
      return query_frustum(t->s, planes, planes_per_query, nq, tol, algo, r, mem, (cudaStream_t)stream, qt);
    });
  }

  int otg_forest_ray_all(const otg_tree* t, const void* rays, const uint64_t* query_offsets, double tol, double tol_increment, double max_distance, int algo,
                         otg_result** out, int mem, void* stream)
  {
    return forest_query(t, query_offsets, out, stream, [&](ResultState& r, u64 nq, const u32* qt) {
      return query_ray(t->s, rays, nq, tol, tol_increment, max_distance, false, algo, r, mem, (cudaStream_t)stream, qt);
    });
  }

  int otg_forest_ray_first(const otg_tree* t, const void* rays, const uint64_t* query_offsets, double tol, double tol_increment, double max_distance,
                           int algo, otg_result** out, int mem, void* stream)
  {
    return forest_query(t, query_offsets, out, stream, [&](ResultState& r, u64 nq, const u32* qt) {
      return query_ray(t->s, rays, nq, tol, tol_increment, max_distance, true, algo, r, mem, (cudaStream_t)stream, qt);
    });
  }

  int otg_autotune_enable(int on)
  {
    tune_enable(on != 0);
    return OTG_OK;
  }

  int otg_autotune_count(void) { return tune_count(); }

  int otg_autotune_force_shape(int shape)
  {
    tune_force(shape);
    return OTG_OK;
  }

  int otg_autotune_entry(int index, char* text, int capacity)
  {
    if (!text || capacity <= 0 || index < 0 || index >= tune_count())
      return OTG_ERR_INVALID_ARGUMENT;
    const std::string s = tune_entry(index);
    std::strncpy(text, s.c_str(), size_t(capacity) - 1);
    text[capacity - 1] = 0;
    return OTG_OK;
  }

  int otg_result_info(const otg_result* r, uint64_t* nq, uint64_t* nids, int* has_distances)
  {
    if (!r)
      return OTG_ERR_INVALID_ARGUMENT;
    if (nq)
      *nq = r->s.nq;
    if (nids)
      *nids = r->s.nids;
    if (has_distances)
      *has_distances = r->s.hasDist ? 1 : 0;
    return OTG_OK;
  }

  int otg_result_copy(const otg_result* r, uint64_t* offsets, uint32_t* ids, double* distances, int mem, void* stream)
  {
    if (!r)
      return OTG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = (cudaStream_t)stream;
    cudaMemcpyKind kind = mem == OTG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    cudaError_t e = cudaSuccess;
    if (offsets)
      e = cudaMemcpyAsync(offsets, r->s.offsets.p, sizeof(uint64_t) * (r->s.nq + 1), kind, st);
    if (!e && ids && r->s.nids)
      e = cudaMemcpyAsync(ids, r->s.ids.p, sizeof(uint32_t) * r->s.nids, kind, st);
    if (!e && distances && r->s.hasDist && r->s.nids)
      e = cudaMemcpyAsync(distances, r->s.dist.p, sizeof(double) * r->s.nids, kind, st);
    if (!e && mem == OTG_MEM_HOST)
      e = cudaStreamSynchronize(st);
    return cuda_status(e, "copying result");
  }

  int otg_result_device_ptrs(const otg_result* r, const uint64_t** offsets, const uint32_t** ids, const double** distances)
  {
    if (!r)
      return OTG_ERR_INVALID_ARGUMENT;
    if (offsets)
      *offsets = r->s.offsets.as<uint64_t>();
    if (ids)
      *ids = r->s.ids.as<uint32_t>();
    if (distances)
      *distances = r->s.hasDist ? r->s.dist.as<double>() : nullptr;
    return OTG_OK;
  }

  int otg_result_stats(const otg_result* r, uint64_t* filter_tests, uint64_t* fp64_rechecks)
  {
    if (!r)
      return OTG_ERR_INVALID_ARGUMENT;
    if (filter_tests)
      *filter_tests = r->s.filterTests;
    if (fp64_rechecks)
      *fp64_rechecks = r->s.rechecks;
    return OTG_OK;
  }

  int otg_profile_enable(int on)
  {
    profiler().enabled = on != 0;
    if (!on)
      profiler().reset();
    return OTG_OK;
  }
  int otg_profile_phase_count(void)
  {
    int n = int(profiler().events.size());
    return n > 0 ? n - 1 : 0;
  }
  int otg_profile_phase(int i, char* name, int cap, float* ms)
  {
    Profiler& p = profiler();
    if (i < 0 || i + 1 >= int(p.events.size()))
      return OTG_ERR_INVALID_ARGUMENT;
    if (name && cap > 0)
    {
      std::strncpy(name, p.names[i].c_str(), size_t(cap - 1));
      name[cap - 1] = 0;
    }
    if (ms)
      return cuda_status(cudaEventElapsedTime(ms, p.events[i], p.events[i + 1]), "reading profile events");
    return OTG_OK;
  }

  void otg_result_free(otg_result* r)
  {
    if (!r)
      return;
    // in stream order on the legacy default stream (the query's own stream may be gone by now)
    r->s.offsets.release_async(nullptr);
    r->s.ids.release_async(nullptr);
    r->s.dist.release_async(nullptr);
    delete r;
  }
}
