// otg_internal.h — host-side state of a GPU tree and of a query result.
//
// HBM layout of a tree with N entities and M nodes (T = double or float):
//   entities     T[N*W]     the caller's entities in input order (W = 3 points, 6 boxes)
//   sortedIds    u32[N]     entity ids in tree (Morton key) order — node entity lists are
//                           contiguous runs of this array, and every subtree is one run
//   sortedGeom   T[N*W]     entities in tree order, so a node's entities are one coalesced read
//   sortedKeys   K[N]       location keys in tree order (K = u32 when they fit in 32 bits)
//   nodeLink     uint4[M]   {firstChild | childCount << 28, ownBegin, ownEnd, subtreeEnd}
//   nodeKey      u64[M]     node key with sentinel bit
//   nodeBox      T[M*6]     {min xyz, size xyz} exactly as GetNodeMinPoint / GetNodeSize
//   nodeMax      T[M*3]     exact max corner of box-tree MBRs (for conservative pruning)
//   nodeDepth    u8[M]
//   nodeParent   u32[M]     (box trees) parent node index
//   ownerNode    u32[N]     (box trees) node that holds the entity at each sorted position
// Nodes are stored breadth-first; the children of a node are contiguous.
#pragma once

#include "../../include/octree_gb300.h"
#include "otg_device.cuh"

#include <cuda_runtime.h>
#include <functional>
#include <string>
#include <utility>
#include <vector>

namespace otg
{

void keep_pool_memory(int device);

// Owning device allocation (move-only; freed on destruction). `ensure` allocates with cudaMalloc;
// `ensure_pooled` allocates in stream order from the device's default memory pool (which keeps
// freed blocks for reuse), for arrays that are replaced often, such as a tree's arrays after an
// Insert: a pooled allocation or free costs microseconds where cudaMalloc / cudaFree of hundreds
// of megabytes cost hundreds.
struct DevBuf
{
  void* p = nullptr;
  size_t bytes = 0;
  bool pooled = false;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes), pooled(o.pooled)
  {
    o.p = nullptr;
    o.bytes = 0;
    o.pooled = false;
  }
  DevBuf& operator=(DevBuf&& o) noexcept
  {
    if (this != &o)
    {
      release();
      p = o.p;
      bytes = o.bytes;
      pooled = o.pooled;
      o.p = nullptr;
      o.bytes = 0;
      o.pooled = false;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  cudaError_t ensure(size_t need)
  {
    if (need <= bytes)
      return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, need ? need : 16);
    if (e == cudaSuccess)
      bytes = need ? need : 16;
    else
      p = nullptr;
    return e;
  }
  cudaError_t ensure_pooled(size_t need, cudaStream_t st)
  {
    if (need <= bytes)
      return cudaSuccess;
    release_async(st);
    int dev = 0;
    cudaGetDevice(&dev);
    keep_pool_memory(dev);
    cudaError_t e = cudaMallocAsync(&p, need ? need : 16, st);
    if (e == cudaSuccess)
    {
      bytes = need ? need : 16;
      pooled = true;
    }
    else
      p = nullptr;
    return e;
  }
  // freed after the work queued on st (a cudaMalloc allocation is freed at once)
  void release_async(cudaStream_t st)
  {
    if (p)
    {
      if (pooled)
        cudaFreeAsync(p, st);
      else
        cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    pooled = false;
  }
  // a pooled allocation is freed after all work on the device, as cudaFree does for the others
  void release()
  {
    if (p)
    {
      if (pooled)
      {
        cudaDeviceSynchronize();
        cudaFreeAsync(p, nullptr);
      }
      else
        cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    pooled = false;
  }
  template<typename X>
  X* as() const
  {
    return reinterpret_cast<X*>(p);
  }
};

// Per-call device scratch of the query paths, stream ordered (cudaMallocAsync / cudaFreeAsync on the
// call's stream, from the device's default memory pool, which keeps up to 8 GiB of freed blocks for
// reuse): a small batch of queries pays no cudaMalloc / cudaFree, and a block is reused only after the
// work queued before its release on that stream.
struct TmpBuf
{
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t st = nullptr;
  TmpBuf() = default;
  TmpBuf(const TmpBuf&) = delete;
  TmpBuf& operator=(const TmpBuf&) = delete;
  ~TmpBuf() { release(); }
  cudaError_t ensure(size_t need, cudaStream_t stream)
  {
    if (need <= bytes)
      return cudaSuccess;
    release();
    int dev = 0;
    cudaGetDevice(&dev);
    keep_pool_memory(dev);
    st = stream;
    cudaError_t e = cudaMallocAsync(&p, need ? need : 16, stream);
    if (e == cudaSuccess)
      bytes = need ? need : 16;
    else
      p = nullptr;
    return e;
  }
  void release()
  {
    if (p)
      cudaFreeAsync(p, st);
    p = nullptr;
    bytes = 0;
  }
  template<typename X>
  X* as() const
  {
    return reinterpret_cast<X*>(p);
  }
  friend void swap(TmpBuf& a, TmpBuf& b) noexcept
  {
    std::swap(a.p, b.p);
    std::swap(a.bytes, b.bytes);
    std::swap(a.st, b.st);
  }
};

// ownerNode of an entity that no node reachable from the root holds (a location outside the grid:
// the reference keeps it in a node the root does not link, so no query or collision sees it)
constexpr u32 kNoOwner = 0xffffffffu;
constexpr u32 kChildShift = 28;
constexpr u32 kFirstChildMask = (1u << kChildShift) - 1;

struct TreeState
{
  TreeState() = default;
  TreeState(const TreeState&) = delete;
  TreeState& operator=(const TreeState&) = delete;
  ~TreeState()
  {
    if (side)
      cudaStreamDestroy(side);
    if (fork)
      cudaEventDestroy(fork);
    if (join)
      cudaEventDestroy(join);
  }

  int scalar = OTG_SCALAR_F64;
  int kind = OTG_KIND_POINTS;
  u64 n = 0;
  u32 D = 0;
  u64 maxElem = 16;
  bool keys32 = false;
  bool built = false;
  bool boxGiven = false;
  u64 maxNodes = 0;

  DevBuf entities, sortedIds, sortedGeom, keysA, keysB, valsB;
  DevBuf nodeLink, nodeKey, nodeBox, nodeMax, nodeDepth;
  DevBuf ownerNode; // u32 per sorted position: the node holding that entity (box trees)
  DevBuf nodeParent; // u32 per node (box trees)
  DevBuf levelCount; // u32[64]: nodes per depth, then splitting nodes per depth
  DevBuf splitQueue; // u32: nodes of the current depth that split
  // point builds emit nodes on a second stream beside the gather (created on first use)
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  DevBuf space;      // Space<T>
  DevBuf sortScratch;
  DevBuf err;        // u32 device error bits
  DevBuf bboxBits;   // ordered-bit min/max accumulators
  DevBuf locations;  // u64 per entity (input order), filled on export request
  DevBuf boxDev;     // the given space box (6 scalars)
  DevBuf rasterTab;  // exact rasterisation thresholds (otg_raster.cuh)
  DevBuf minTab;     // MinPoint node table per (dimension, depth, cell)
  // forest: `trees` independent trees built and queried together (0 = a single tree). Node t is
  // the root of tree t; tree t holds the entities [treeOff[t], treeOff[t+1]) of the input.
  u32 trees = 0;
  std::vector<u64> treeOffHost;
  std::vector<u32> treeDHost;
  DevBuf treeOff;    // u64[trees + 1]
  DevBuf treeD;      // u32[trees]: max depth of each tree
  DevBuf nodeTree;   // u32 per node: its tree
  DevBuf tabOff;     // u64[trees + 1]: offset of each tree's threshold tables (entries)
  DevBuf minOff;     // u64[trees + 1]: offset of each tree's MinPoint table (point trees)
  DevBuf segTiles;   // uint2 per sort tile: {tree, tile within the tree}
  std::vector<u64> tabOffHost, minOffHost;
  std::vector<uint2> segTilesHost;
  // static linear layout (otg_static.cu), filled by export_static: the dynamic node of each static
  // node, then the reference's arrays, and the per-level control block
  DevBuf stOrder, stChildBegin, stSeg, stDepth, stGeom, stCtl;
  DevBuf geom32;     // FP32 image of sortedGeom for the query filters (built on first use)
  DevBuf nodeBox32;  // FP32 outward-rounded node boxes for the query filters
  bool image32 = false;
  // a bulk Insert changed the tree: nodes may own entities beside their children and child links
  // may skip levels, which the static array layout cannot hold
  bool inserted = false;
  // arrays an Insert replaced that were allocated with cudaMalloc: kept until the next Create or the
  // tree's end, so that the Insert itself waits for no cudaFree
  std::vector<DevBuf> retired;

  // cached after the build (host copies, filled by sync)
  u64 nodeCount = 0;
  bool countsKnown = false;
  std::vector<u32> levelCountsHost;

  const void* sortedKeys = nullptr; // final sorted keys (keysA or keysB)
};

struct ResultState
{
  u64 nq = 0;
  u64 nids = 0;
  bool hasDist = false;
  // the arrays come from the stream-ordered pool on the query's stream and go back to it in that
  // stream's order (result_alloc, otg_result_free)
  cudaStream_t stream = nullptr;
  DevBuf offsets; // u64[nq+1]
  DevBuf ids;     // u32[nids]
  DevBuf dist;    // double[nids]
  ResultState() = default;
  ResultState(const ResultState&) = delete;
  ResultState& operator=(const ResultState&) = delete;
  ~ResultState()
  {
    offsets.release_async(stream);
    ids.release_async(stream);
    dist.release_async(stream);
  }
  u64 filterTests = 0;
  u64 rechecks = 0;
};

void set_error(const std::string& msg);

// build-phase instrumentation (otg_capi.cu): mark() records an event on the stream when enabled
struct Profiler
{
  bool enabled = false;
  std::vector<std::string> names;
  std::vector<cudaEvent_t> events;
  void reset();
  void mark(const char* name, cudaStream_t st);
};
Profiler& profiler();
int cuda_status(cudaError_t e, const char* what);
// a query result's arrays (bytes of each; 0 leaves one unallocated), from the pool on stream st
inline cudaError_t result_alloc(ResultState& r, size_t offBytes, size_t idBytes, size_t distBytes, cudaStream_t st)
{
  r.stream = st;
  cudaError_t e = cudaSuccess;
  if (offBytes && (e = r.offsets.ensure_pooled(offBytes, st)))
    return e;
  if (idBytes && (e = r.ids.ensure_pooled(idBytes, st)))
    return e;
  if (distBytes && (e = r.dist.ensure_pooled(distBytes, st)))
    return e;
  return cudaSuccess;
}

// kernel-shape autotuner (otg_tune.cu): runs launch(shape) with the fastest candidate shape of the
// key's size class, timing every candidate on the first call of the class
std::string tune_key(const char* op, bool f64, int kind, u64 entities, u64 queries);
int tune_run(const std::string& key, const std::vector<std::pair<int, const char*>>& cands, int fallback, cudaStream_t st,
             const std::function<int(int)>& launch);
int tune_lookup(const std::string& key, int fallback);
void tune_enable(bool on);
void tune_force(int shape); // -1: none
int tune_count();
std::string tune_entry(int i);

// build entry (otg_build.cu)
int build_tree(TreeState& t, const void* entities, u64 n, u32 maxDepth, const void* box, u64 maxElem, int mem, cudaStream_t st);
int build_forest(TreeState& t, const void* entities, const u64* treeOffsets, u32 trees, u32 maxDepth, const void* boxes, u64 maxElem, int mem,
                 cudaStream_t st);
int finish_build(TreeState& t, cudaStream_t st);
int set_entities(TreeState& t, const void* entities, u64 n, int mem, cudaStream_t st);
int insert_points(TreeState& t, const void* entities, u64 n, int mem, cudaStream_t st);
int forest_relaunch(TreeState& t, const void* entities, const void* boxes, cudaStream_t st);
int export_locations(const TreeState& t, u64* keys, int mem, cudaStream_t st);
int export_nodes(const TreeState& t, u64* keys, double* minSize, u64* eoff, u32* eids, u32* childCount);
// the static linear layout of a single tree (otg_static.cu)
int export_static(TreeState& t, otg_static_layout* out, cudaStream_t st);
// the reference's binary archive of that static tree, and a tree resumed from one (otg_archive.cu)
int save_static_archive(TreeState& t, bool managed, void* buffer, u64 capacity, u64* size, cudaStream_t st);
int load_static_archive(TreeState& t, const void* buffer, u64 size, const void* box, cudaStream_t st);

// queries (otg_query.cu). qTree: the tree of each query when t is a forest (null otherwise).
int query_range(const TreeState& t, const void* ranges, u64 nq, int mode, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                const u32* qTree = nullptr);
int query_pick(const TreeState& t, const void* pts, u64 nq, double tol, int algo, ResultState& r, int mem, cudaStream_t st, const u32* qTree = nullptr);
int query_knn(const TreeState& t, const void* pts, u64 nq, const u32* k, u32 kAll, double maxDist, double tol, int algo, ResultState& r, int mem,
              cudaStream_t st, const u32* qTree = nullptr);
// combined queries (otg_query): conds in the otg_condition layout, query q holds [off[q], off[q + 1])
int query_combined(const TreeState& t, const void* conds, const u64* off, u64 nq, const void* planes, const unsigned char* cross, u64 nPlanes,
                   const void* boxes, u64 nBoxes, int orOp, double tol, int algo, ResultState& r, int mem, cudaStream_t st);
// one plane {origoDistance, nx, ny, nz} per query: PlaneSearch, or PlanePositiveSegmentation (positive)
int query_plane(const TreeState& t, const void* planes, u64 nq, bool positive, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                const u32* qTree = nullptr);
int query_frustum(const TreeState& t, const void* planes, u64 np, u64 nq, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                  const u32* qTree = nullptr);
int query_ray(const TreeState& t, const void* rays, u64 nq, double tol, double tolInc, double maxDist, bool first, int algo, ResultState& r,
              int mem, cudaStream_t st, const u32* qTree = nullptr);
// per-query trees of a forest from host query offsets (queries [qoff[t], qoff[t+1]) ask tree t)
int forest_query_trees(const TreeState& t, const u64* qoffHost, DevBuf& qoffDev, DevBuf& qTree, u64& nq, cudaStream_t st);
int query_collide_self(const TreeState& t, double tol, int algo, ResultState& r, cudaStream_t st);
int query_collide_pair(const TreeState& a, const TreeState& b, double tol, int algo, ResultState& r, cudaStream_t st);
// batched filtered kNN on point trees (otg_knn.cu); inputs in device memory
int knn_filtered(TreeState& t, const void* dpts, const u32* dk, u64 nq, u32 kAll, double maxDist, double tol, ResultState& r, cudaStream_t st);
// kNN into caller-owned slots with static scratch: allocates no memory
int query_knn_noalloc(const TreeState& t, const void* pts, u64 nq, u32 k, double maxDist, double tol, u32 cap, u32* counts, u32* ids, double* dist,
                      cudaStream_t st);

} // namespace otg

// the opaque handles of the C-ABI
struct otg_tree
{
  otg::TreeState s;
};
struct otg_result
{
  otg::ResultState s;
};
