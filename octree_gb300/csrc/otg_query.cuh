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
  DevBuf k1, v1, scratch;
  cudaError_t e;
  if ((e = k1.ensure(sizeof(u64) * m)) || (e = v1.ensure(sizeof(u32) * m)) || (e = scratch.ensure(SortScratch::bytes(m, passes))))
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
  cudaStreamSynchronize(st);
  k1.release();
  v1.release();
  scratch.release();
  return cuda_status(cudaGetLastError(), "sorting results");
}

static inline int sort_pairs_u32(u32* keys, u32* vals, u64 m, u32 bits, cudaStream_t st, u32* err)
{
  if (m <= 1 || bits == 0)
    return OTG_OK;
  const u32 passes = (bits + kRadixBits - 1) / kRadixBits;
  DevBuf k1, v1, scratch;
  cudaError_t e;
  if ((e = k1.ensure(sizeof(u32) * m)) || (e = v1.ensure(sizeof(u32) * m)) || (e = scratch.ensure(SortScratch::bytes(m, passes))))
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
  cudaStreamSynchronize(st);
  k1.release();
  v1.release();
  scratch.release();
  return cuda_status(cudaGetLastError(), "sorting results");
}

// qTree: the tree of each query when t is a forest (null for a single tree)
template<typename T>
static inline TreeView<T> view(const TreeState& t, const u32* qTree = nullptr)
{
  return TreeView<T>{ t.nodeLink.as<uint4>(), t.nodeBox.as<T>(), t.nodeMax.as<T>(), t.sortedIds.as<u32>(), t.sortedGeom.as<T>(), u32(t.n),
                      t.kind == OTG_KIND_BOXES ? 1 : 0, u32(t.nodeCount), qTree, qTree ? t.treeOff.as<u64>() : nullptr };
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
int batch_range(const TreeView<T>& tv, const T* ranges, u32 nq, int mode, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape = 4);
template<typename T>
int batch_frustum(const TreeView<T>& tv, const T* planes, u32 np, u32 nq, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape = 4);
template<typename T>
int batch_plane(const TreeView<T>& tv, const T* planes, u32 nq, bool positive, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape = 4);
template<typename T>
int batch_ray_all(const TreeView<T>& tv, const T* rays, u32 nq, T tol, T tolInc, T maxDist, Appender out, u32* work, u32* err, cudaStream_t st,
                  int shape = 4);

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
