// otg_query.cuh — pieces shared by the query translation units: the device view of a built tree,
// the result appender, the reference's distance helpers, and host helpers for sorting results.
#pragma once

#include "otg_internal.h"
#include "otg_sort.cuh"

#include <algorithm>
#include <cmath>

namespace otg
{

constexpr int kStack = 168; // > 7 * 19 + 1 entries: depth-first stack bound for maxDepth <= 19

template<typename T>
struct TreeView
{
  const uint4* link;
  const T* nodeBox; // {min xyz, size xyz}
  const T* nodeMax; // box trees: exact max corner
  const u32* ids;   // sortedIds
  const T* geom;    // sortedGeom
  u32 n;
  int isBox;
  u32 nNodes;
  const u32* qTree;   // forest: tree (= root node) of each query; null for a single tree
  const u64* treeOff; // forest: first entity of each tree (ids are returned relative to it)
  const unsigned char* nodeDepth; // depth of each node below its tree's root
  // FP32 images (point trees of FP64 entities, built on demand): outward-rounded node boxes (two
  // float4 per node) and round-to-nearest entities; null where a kernel takes the FP64 tests only
  const float4* nodeImg = nullptr;
  const float4* pointImg = nullptr;
};

// root node and id base of query q (node t is the root of tree t in a forest)
template<typename T>
__device__ __forceinline__ u32 query_root(const TreeView<T>& tv, u32 q)
{
  return tv.qTree ? tv.qTree[q] : 0u;
}
template<typename T>
__device__ __forceinline__ u32 id_base(const TreeView<T>& tv, u32 root)
{
  return tv.qTree ? u32(tv.treeOff[root]) : 0u;
}

struct Appender
{
  u64* items;      // (query << 32) | id
  double* dist;    // optional
  unsigned long long* count;
  u64 capacity;
  __device__ __forceinline__ void put(u32 q, u32 id, double d = 0.0)
  {
    u64 pos = atomicAdd(count, 1ull);
    if (pos < capacity)
    {
      items[pos] = (u64(q) << 32) | id;
      if (dist)
        dist[pos] = d;
    }
  }
  __device__ __forceinline__ u64 reserve(u64 len) { return atomicAdd(count, (unsigned long long)len); }
};

// ---- combined queries (core/ot_query.h:835-1026): conditions of the otg_condition layout
struct QueryCond
{
  int kind;
  u32 first;
  u32 count;
  u32 reserved;
  double tol;
};
constexpr int kCondFrustum = OTG_COND_FRUSTUM, kCondRangeInside = OTG_COND_RANGE_INSIDE, kCondRangeOverlap = OTG_COND_RANGE_OVERLAP,
              kCondPlane = OTG_COND_PLANE;

template<typename T>
struct QueryProgram
{
  const QueryCond* conds;
  const u64* off;    // conditions of query q: [off[q], off[q + 1])
  const T* planes;   // {origo distance, normal} per plane
  const unsigned char* cross; // isCrossingAllowed per plane
  const T* boxes;
  u64 nConds, nPlanes, nBoxes;
  int orOp;
};

// whether condition c names planes / a box inside the arrays (a bad one reads nothing)
template<typename T>
__device__ __forceinline__ bool cond_valid(const QueryProgram<T>& qp, const QueryCond& c)
{
  if (c.kind == kCondFrustum)
    return u64(c.first) + c.count <= qp.nPlanes;
  if (c.kind == kCondPlane)
    return c.first < qp.nPlanes;
  if (c.kind == kCondRangeInside || c.kind == kCondRangeOverlap)
    return c.first < qp.nBoxes;
  return false;
}

// ot_query.h:893-916: node selection of one condition (node {min xyz, size xyz})
template<typename T>
__device__ __forceinline__ bool cond_node(const QueryProgram<T>& qp, const QueryCond& c, const T* nb, T tol)
{
  using G = GeoD<T>;
  if (c.kind == kCondFrustum)
  {
    for (u32 i = c.first; i < c.first + c.count; ++i)
    {
      const int rel = G::box_plane(nb, nb + 3, qp.planes[4 * u64(i)], qp.planes + 4 * u64(i) + 1, tol);
      if (rel == 1)
        return true;
      if (rel == 0)
        return false;
    }
    return true;
  }
  if (c.kind == kCondPlane)
  {
    const T ptol = c.tol < 0 ? base_tol<T>() : T(c.tol);
    return G::box_plane(nb, nb + 3, qp.planes[4 * u64(c.first)], qp.planes + 4 * u64(c.first) + 1, ptol) == 1;
  }
  const T* r = qp.boxes + 6 * u64(c.first);
  T rsize[3] = { T(r[3] - r[0]), T(r[4] - r[1]), T(r[5] - r[2]) };
  T nmin[3] = { nb[0], nb[1], nb[2] }, nsize[3] = { nb[3], nb[4], nb[5] };
  return G::overlap_by_min_point(r, rsize, nmin, nsize, tol);
}

// ot_query.h:949-998: entity selection of one condition (g: the entity's point or box)
template<typename T>
__device__ __forceinline__ bool cond_entity(const QueryProgram<T>& qp, const QueryCond& c, const T* g, bool isBox, T tol)
{
  using G = GeoD<T>;
  auto rel = [&](const T* pl, T t) {
    if (isBox)
    {
      T bsize[3] = { T(g[3] - g[0]), T(g[4] - g[1]), T(g[5] - g[2]) };
      return G::box_plane(g, bsize, pl[0], pl + 1, t);
    }
    return G::point_plane(g, pl[0], pl + 1, t);
  };
  if (c.kind == kCondFrustum)
  {
    for (u32 i = c.first; i < c.first + c.count; ++i)
    {
      const int r = rel(qp.planes + 4 * u64(i), tol);
      if (r == 0 || (r == 1 && !qp.cross[i]))
        return false;
    }
    return true;
  }
  if (c.kind == kCondPlane)
    return rel(qp.planes + 4 * u64(c.first), c.tol < 0 ? base_tol<T>() : T(c.tol)) == 1;
  T r[6];
#pragma unroll
  for (int k = 0; k < 6; ++k)
    r[k] = qp.boxes[6 * u64(c.first) + k];
  if (!isBox)
    return G::box_contains_point(r, g, tol);
  return c.kind == kCondRangeInside ? G::contains_box_no_tol(r, g) : G::box_relation(r, g, tol) == -1;
}

// the conditions of query q over a node (node) or an entity (entity): all of them (And) or any (Or);
// no condition passes every node and entity under And and none under Or
template<typename T, typename F>
__device__ __forceinline__ bool cond_combine(const QueryProgram<T>& qp, u32 q, u32* err, F&& test)
{
  const u64 c0 = qp.off[q], c1 = qp.off[q + 1];
  if (c1 < c0 || c1 > qp.nConds)
  {
    atomicOr(err, kErrArgument);
    return false;
  }
  for (u64 i = c0; i < c1; ++i)
  {
    const QueryCond c = qp.conds[i];
    if (!cond_valid(qp, c))
    {
      atomicOr(err, kErrArgument);
      return false;
    }
    const bool ok = test(c);
    if (qp.orOp && ok)
      return true;
    if (!qp.orOp && !ok)
      return false;
  }
  return !qp.orOp;
}

template<typename T>
__device__ __forceinline__ void load_box(const T* p, T b[6])
{
#pragma unroll
  for (int c = 0; c < 6; ++c)
    b[c] = p[c];
}

// ot_query.h:1033-1036 GetValueWithToleranceUpper
template<typename T>
__device__ __forceinline__ T upper_tol(T v, T tol)
{
  return fmax(tol, v * (T(1.0) + tol));
}

template<typename T>
__device__ __forceinline__ T entity_distance(const TreeView<T>& tv, u32 e, const T* p, T tol)
{
  if (tv.isBox)
  {
    T mn, mm;
    GeoD<T>::min_max_distance(p, tv.geom + u64(e) * 6, tol, mn, mm);
    return mn;
  }
  return GeoD<T>::distance(p, tv.geom + u64(e) * 3);
}

constexpr int kKnnMaxK = 256;

// u64 offsets from u32 counts (otg_knn.cu): per-tile sums, their scan in one block (the grand total
// at tileSums[tiles]), and the offsets; off holds n + 1 entries
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const u32* __restrict__ cnt, u64 n, u64* __restrict__ tileSums);
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(u64* __restrict__ tileSums, u64 tiles);
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const u32* __restrict__ cnt, u64 n, const u64* __restrict__ tileSums,
                                                                  u64* __restrict__ off);
static inline int blocks_for(u64 n, int per = 256)
{
  return int(std::max<u64>(1, std::min<u64>((n + per - 1) / per, 152 * 16)));
}

static inline u32 bit_count(u64 v)
{
  u32 b = 0;
  while (v)
  {
    ++b;
    v >>= 1;
  }
  return b;
}

// Stable radix sort of (u64 key, u32 value) with temporary buffers; result in (keys, vals).
static inline int sort_pairs_u64(u64* keys, u32* vals, u64 m, u32 bits, cudaStream_t st, u32* err)
{
  if (m <= 1 || bits == 0)
    return OTG_OK;
  const u32 passes = (bits + kRadixBits - 1) / kRadixBits;
  TmpBuf k1, v1, scratch;
  cudaError_t e;
  if ((e = k1.ensure(sizeof(u64) * m, st)) || (e = v1.ensure(sizeof(u32) * m, st)) || (e = scratch.ensure(SortScratch::bytes(m, passes), st)))
    return cuda_status(e, "allocating sort buffers");
  cudaMemsetAsync(scratch.p, 0, SortScratch::bytes(m, passes), st);
  SortScratch ss;
  ss.carve(scratch.p, m, passes);
  radix_histogram_kernel<u64><<<blocks_for(m), 256, 0, st>>>(keys, m, 0, passes, ss.hist);
  bool inB = onesweep_passes<u64>(keys, vals, k1.as<u64>(), v1.as<u32>(), m, 0, passes, false, ss, err, st);
  if (inB)
  {
    cudaMemcpyAsync(keys, k1.p, sizeof(u64) * m, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(vals, v1.p, sizeof(u32) * m, cudaMemcpyDeviceToDevice, st);
  }
  // the scratch is released in stream order after the copies above
  return cuda_status(cudaGetLastError(), "sorting results");
}

static inline int sort_pairs_u32(u32* keys, u32* vals, u64 m, u32 bits, cudaStream_t st, u32* err)
{
  if (m <= 1 || bits == 0)
    return OTG_OK;
  const u32 passes = (bits + kRadixBits - 1) / kRadixBits;
  TmpBuf k1, v1, scratch;
  cudaError_t e;
  if ((e = k1.ensure(sizeof(u32) * m, st)) || (e = v1.ensure(sizeof(u32) * m, st)) || (e = scratch.ensure(SortScratch::bytes(m, passes), st)))
    return cuda_status(e, "allocating sort buffers");
  cudaMemsetAsync(scratch.p, 0, SortScratch::bytes(m, passes), st);
  SortScratch ss;
  ss.carve(scratch.p, m, passes);
  radix_histogram_kernel<u32><<<blocks_for(m), 256, 0, st>>>(keys, m, 0, passes, ss.hist);
  bool inB = onesweep_passes<u32>(keys, vals, k1.as<u32>(), v1.as<u32>(), m, 0, passes, false, ss, err, st);
  if (inB)
  {
    cudaMemcpyAsync(keys, k1.p, sizeof(u32) * m, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(vals, v1.p, sizeof(u32) * m, cudaMemcpyDeviceToDevice, st);
  }
  // the scratch is released in stream order after the copies above
  return cuda_status(cudaGetLastError(), "sorting results");
}

// qTree: the tree of each query when t is a forest (null for a single tree)
template<typename T>
static inline TreeView<T> view(const TreeState& t, const u32* qTree = nullptr)
{
  return TreeView<T>{ t.nodeLink.as<uint4>(), t.nodeBox.as<T>(), t.nodeMax.as<T>(), t.sortedIds.as<u32>(), t.sortedGeom.as<T>(), u32(t.n),
                      t.kind != OTG_KIND_POINTS ? 1 : 0, u32(t.nodeCount), qTree, qTree ? t.treeOff.as<u64>() : nullptr,
                      t.nodeDepth.as<unsigned char>() };
}

template<typename T>
static inline T upper_tol_host(T v, T tol)
{
  return std::fmax(tol, v * (T(1.0) + tol));
}

template<typename T>
static inline T tol_of(double tol)
{
  return tol < 0 ? base_tol<T>() : T(tol);
}

// batched warp-per-query kernels (otg_batch.cu); `work` is a device counter the launch resets;
// shape: warps per block (2, 4 or 8)
template<typename T>
int batch_range(const TreeView<T>& tv, const T* ranges, u32 nq, int mode, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape = 4, size_t workBytes = 0);
// Work buffer of the batched kernels: four counters, then the (query, subtree) items of a split
// batch. A split batch runs in two launches: each query runs its levels above the split depth, and
// the subtrees at the split depth that it enters become items that any warp takes, so that a few
// costly queries (large trees of a forest, wide frusta) spread over the whole GPU.
// The split depth is part of a batched kernel's shape (shape = warps per block | code << 8):
//   code 0: the default, depth 2 for batches of at most kSplitQueries queries, else no split;
//   code 1: no split; code 2, 3, 4: split depth 1, 2, 3.
// The autotuner chooses among the depths that the batch's size allows (split_depth_limit).
constexpr u32 kSplitQueries = 8192;
constexpr u32 kSplitDefaultDepth = 2;
constexpr u32 kSplitMaxQueries = 65536;
inline u64 split_items_per_query(u32 depth) { return u64(1) << (3 * depth); }
// deepest split a batch of nq queries may use (its items fit 32 MB): 3 up to 8192 queries, 2 up to
// 65536, else none
inline u32 split_depth_limit(u64 nq) { return nq <= kSplitQueries ? 3u : nq <= kSplitMaxQueries ? 2u : 0u; }
inline size_t batch_work_bytes(u64 nq)
{
  const u32 d = split_depth_limit(nq);
  return 16 + (d ? sizeof(u64) * split_items_per_query(d) * nq : 0);
}
// split depth (0: none) of a shape for a batch of nq queries
inline u32 shape_split_depth(int shape, u64 nq)
{
  const int code = shape >> 8;
  const u32 d = code == 0 ? (nq <= kSplitQueries ? kSplitDefaultDepth : 0u) : u32(code - 1);
  return d <= split_depth_limit(nq) ? d : 0u;
}
template<typename T>
int batch_frustum(const TreeView<T>& tv, const T* planes, u32 np, u32 nq, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape = 4, size_t workBytes = 0);
template<typename T>
int batch_plane(const TreeView<T>& tv, const T* planes, u32 nq, bool positive, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape = 4, size_t workBytes = 0);
template<typename T>
int batch_pick(const TreeView<T>& tv, const T* pts, u32 nq, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape = 4, size_t workBytes = 0);
template<typename T>
int batch_query_program(const TreeView<T>& tv, const QueryProgram<T>& qp, u32 nq, T tol, Appender out, u32* work, u32* err, cudaStream_t st,
                        int shape = 4, size_t workBytes = 0);
template<typename T>
int batch_ray_all(const TreeView<T>& tv, const T* rays, u32 nq, T tol, T tolInc, T maxDist, Appender out, u32* work, u32* err, cudaStream_t st,
                  int shape = 4, size_t workBytes = 0);

// autotuner size class of a batched query
inline std::string query_key(const char* op, int algo, bool forest, bool f64, int kind, u64 n, u64 nq)
{
  std::string name = std::string(op) + (forest ? " forest" : "") + (algo == OTG_ALGO_FILTERED ? " warp" : "");
  return tune_key(name.c_str(), f64, kind, n, nq);
}

// FP32 images of a built tree for the query filters (otg_knn.cu): built on first use after a build
int ensure_image32(TreeState& t, cudaStream_t st);

// filtered candidate search of CollisionDetection (otg_collide.cu)
struct CollideSearch
{
  DevBuf imgA, imgB, ctr; // tolerance-specific FP32 box images, counters
  DevBuf order;           // processing order of the first tree's entities
  DevBuf nodesB;          // the second tree's node MBRs with the tolerance added
  float tolHi = 0.f;
  bool ready = false;
  bool orderReady = false;
};
int collide_search_filtered(TreeState& A, TreeState& B, bool self, double tol, Appender out, u32* err, CollideSearch& s, cudaStream_t st);
int collide_search_stats(const CollideSearch& s, u64& tests, u64& rechecks, cudaStream_t st);

} // namespace otg
