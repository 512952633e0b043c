// otg_static.cu — a built tree in the array layout of the reference's StaticLinearOrthoTreeCore
// (core/ot_static_linear_core.h), computed on the device from the dynamic tree's nodes.
//
// The static tree is the dynamic tree with its pass-through nodes contracted. A node below the
// root with exactly one child and no entities of its own holds the same entities as that child.
// The reference's static Build (:419-521) turns each child group into one node placed at the
// lowest common ancestor of the group's locations (detail/si_morton.h:347-387). That ancestor is
// the first node down the pass-through chain that either splits its entities two ways or keeps
// some of them (a node at depth d whose entities differ in the digit of level d + 1, or one of
// which has depth d). A leaf sits at the lowest common ancestor of its own locations, which can be
// below its dynamic depth. The root stays at depth 0 even when it passes everything through.
//
// Nodes are numbered breadth first by static level, children in Morton order: the queue order of
// Build over sorted locations. One step per static level, three launches each, with nothing read
// back between levels:
//   static_count_kernel   child count of each node of the level, summed per block
//   static_scan_kernel    exclusive scan of the block sums; size and start of the next level
//   static_assign_kernel  per node: child segment begin (next level start + scan), entity segment,
//                         depth and MinPoint; per child: the dynamic node at the end of the
//                         pass-through chain below the dynamic child becomes the next level's node
// MBR geometry (box trees) then goes up one level per launch: a node's own entities, then its
// children's min + size, as InitializeMinimalNodeGeometry (:281-325) unites them.
#include "otg_internal.h"

namespace otg
{
namespace
{

constexpr u32 kStaticBlocks = 304; // two per SM; a level is split into this many contiguous chunks
constexpr u32 kStaticThreads = 256;
constexpr u32 kMaxLevels = 40;     // static levels <= max depth + 1 <= 22
constexpr u32 kErrChain = 1u;      // a pass-through chain longer than any tree can hold
constexpr u32 kErrOrder = 2u;      // more static nodes than dynamic ones

struct StaticCtl
{
  u32 levelStart[kMaxLevels];
  u32 levelCount[kMaxLevels];
  u32 blockSum[kStaticBlocks];
  unsigned long long covered; // entities in some node's entity segment
  u32 lastParentPlus1;        // highest node id with children + 1 (0: no node has children)
  u32 err;
};

__device__ __forceinline__ u32 child_count(const uint4& L) { return L.x >> kChildShift; }

// a node below the root that only hands its entities to its single child
__device__ __forceinline__ bool pass_through(const uint4& L) { return child_count(L) == 1u && L.z == L.y; }

__device__ __forceinline__ u32 bit_width64(u64 v) { return v ? 64u - u32(__clzll((long long)v)) : 0u; }

// this block's contiguous part [b, e) of level l, whose nodes start at id `start`; clamped to the
// `cap` node slots (static nodes are a subset of the dynamic ones, so only inconsistent links could
// ask for more, and those set kErrOrder where they are written)
__device__ __forceinline__ void level_chunk(const StaticCtl* c, u32 l, u32 cap, u32& start, u32& b, u32& e)
{
  start = min(c->levelStart[l], cap);
  const u32 cnt = min(c->levelCount[l], cap - start);
  const u32 per = (cnt + gridDim.x - 1) / gridDim.x;
  b = min(cnt, blockIdx.x * per);
  e = min(cnt, b + per);
}

// block-wide sum (every thread gets it)
__device__ __forceinline__ u64 block_sum(u64 v)
{
  __shared__ u64 warpSums[kStaticThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1)
    v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0)
    warpSums[warp] = v;
  __syncthreads();
  u64 t = 0;
  for (int w = 0; w < int(blockDim.x >> 5); ++w)
    t += warpSums[w];
  return t;
}

// block-wide exclusive scan of v; total gets the block's sum
__device__ __forceinline__ u32 block_exclusive_scan(u32 v, u32& total)
{
  __shared__ u32 warpTot[kStaticThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const u32 y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o)
      incl += y;
  }
  __syncthreads();
  if (lane == 31)
    warpTot[warp] = incl;
  __syncthreads();
  u32 before = 0;
  total = 0;
  for (int w = 0; w < int(blockDim.x >> 5); ++w)
  {
    const u32 s = warpTot[w];
    before += (w < warp) ? s : 0u;
    total += s;
  }
  return before + incl - v;
}

__global__ void static_init_kernel(StaticCtl* c, u32* order)
{
  for (u32 i = threadIdx.x; i < kMaxLevels; i += blockDim.x)
  {
    c->levelStart[i] = 0;
    c->levelCount[i] = i == 0 ? 1u : 0u;
  }
  if (threadIdx.x == 0)
  {
    c->covered = 0;
    c->lastParentPlus1 = 0;
    c->err = 0;
    order[0] = 0; // the root
  }
}

__global__ void __launch_bounds__(kStaticThreads) static_count_kernel(StaticCtl* c, u32 l, const u32* __restrict__ order, const uint4* __restrict__ link,
                                                                     u32 cap)
{
  u32 start, b, e;
  level_chunk(c, l, cap, start, b, e);
  u64 sum = 0;
  for (u32 i = b + threadIdx.x; i < e; i += blockDim.x)
    sum += child_count(link[order[start + i]]);
  sum = block_sum(sum);
  if (threadIdx.x == 0)
    c->blockSum[blockIdx.x] = u32(sum);
}

__global__ void static_scan_kernel(StaticCtl* c, u32 l, u32 blocks)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  u32 run = 0;
  for (u32 b = 0; b < blocks; ++b)
  {
    const u32 v = c->blockSum[b];
    c->blockSum[b] = run;
    run += v;
  }
  c->levelStart[l + 1] = c->levelStart[l] + c->levelCount[l];
  c->levelCount[l + 1] = run;
}

template<typename T, typename K, bool IS_BOX>
__global__ void __launch_bounds__(kStaticThreads) static_assign_kernel(StaticCtl* c, u32 l, const uint4* __restrict__ link,
                                                                      const unsigned char* __restrict__ nodeDepth, const K* __restrict__ keys,
                                                                      u32* __restrict__ order, u32 orderCap, u32* __restrict__ childBegin,
                                                                      uint2* __restrict__ seg, unsigned char* __restrict__ depthOut,
                                                                      T* __restrict__ geom, const T* __restrict__ minTab, u32 D, u64 maxElem)
{
  u32 start, b, e;
  level_chunk(c, l, orderCap, start, b, e);
  const u32 base = c->levelStart[l + 1] + c->blockSum[blockIdx.x];
  const u64 tabPerDim = (u64(2) << D) - 1;
  u32 carry = 0;
  u64 covered = 0;
  for (u32 tile = b; tile < e; tile += blockDim.x)
  {
    const u32 i = tile + threadIdx.x;
    const bool active = i < e;
    const u32 x = active ? order[start + i] : 0u;
    const uint4 L = active ? link[x] : make_uint4(0, 0, 0, 0);
    const u32 cc = active ? child_count(L) : 0u;
    u32 total;
    const u32 excl = block_exclusive_scan(cc, total);
    if (active && L.w <= L.y)
    {
      atomicOr(&c->err, kErrOrder); // every node of a tree with entities holds some
    }
    else if (active)
    {
      const u32 id = start + i;
      const u32 cb = base + carry + excl;
      childBegin[id] = cb;
      // CreateNode (:383-414): a node that splits keeps the entities of its own depth (the stuck
      // run at the front of its range); a leaf keeps its whole range
      const u32 own = cc ? L.z - L.y : L.w - L.y;
      seg[id] = make_uint2(L.y, own);
      covered += own;
      // depth: the root stays at 0; a node that splits is at the lowest common ancestor already
      u32 dep = 0;
      if (x != 0)
      {
        if (cc)
          dep = nodeDepth[x];
        else
        {
          // LowestCommonAncestorCalculator over the leaf's sorted range: the highest differing
          // location bit is the one of its first and last location; boxes also take the least
          // entity depth (points all have depth D)
          const u64 kf = u64(keys[L.y]), kl = u64(keys[L.w - 1]);
          const u64 diff = IS_BOX ? ((kf >> 5) ^ (kl >> 5)) : ((kf - 1) ^ (kl - 1));
          const u32 lcaDepth = D - (bit_width64(diff) + 2) / 3;
          u32 minDepth = D;
          if constexpr (IS_BOX)
          {
            // a leaf above maxElem is at max depth or holds only entities of its own depth
            if (u64(L.w - L.y) > maxElem)
              minDepth = nodeDepth[x];
            else
            {
              minDepth = 31;
              for (u32 j = L.y; j < L.w; ++j)
                minDepth = min(minDepth, u32(u64(keys[j]) & 31u));
            }
          }
          dep = min(minDepth, lcaDepth);
        }
      }
      depthOut[id] = (unsigned char)dep;
      if constexpr (!IS_BOX)
      {
        // InitNodeGeometry (:346-366): the MinPoint of the node at `dep` on the first location
        const u64 locFirst = u64(keys[L.y]) - 1;
        const u64 loc = locFirst >> (3 * (D - dep));
#pragma unroll
        for (int dim = 0; dim < 3; ++dim)
          geom[u64(id) * 3 + dim] = minTab[u64(dim) * tabPerDim + ((u64(1) << dep) - 1) + compact1by2(loc >> dim)];
      }
      if (cc)
      {
        atomicMax(&c->lastParentPlus1, id + 1);
        const u32 fc = L.x & kFirstChildMask;
        for (u32 k = 0; k < cc; ++k)
        {
          u32 y = fc + k;
          bool ended = false;
          for (u32 s = 0; s < 64 && y < orderCap; ++s)
          {
            const uint4 Ly = link[y];
            if (!pass_through(Ly))
            {
              ended = true;
              break;
            }
            y = Ly.x & kFirstChildMask;
          }
          if (!ended)
            atomicOr(&c->err, kErrChain);
          // every slot of the next level is written (the root stands in after an error), so
          // the next level reads only valid node indices
          if (cb + k < orderCap)
            order[cb + k] = ended ? y : 0u;
          else
            atomicOr(&c->err, kErrOrder);
        }
      }
    }
    carry += total;
  }
  covered = block_sum(covered);
  if (threadIdx.x == 0 && covered)
    atomicAdd(&c->covered, (unsigned long long)covered);
}

// the end of the child segment begins: node_count at index node_count (<= cap)
__global__ void static_finish_kernel(StaticCtl* c, u32* childBegin, u32 cap)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  for (u32 l = 0; l < kMaxLevels; ++l)
    if (c->levelCount[l] == 0)
    {
      if (c->levelStart[l] <= cap)
        childBegin[c->levelStart[l]] = c->levelStart[l];
      else
        atomicOr(&c->err, kErrOrder);
      return;
    }
}

// InitializeMinimalNodeGeometry (:281-325), one static level per launch from the deepest up
template<typename T>
__global__ void __launch_bounds__(kStaticThreads) static_mbr_kernel(const StaticCtl* c, u32 l, const u32* __restrict__ childBegin,
                                                                   const uint2* __restrict__ seg, const T* __restrict__ sortedGeom, T* __restrict__ geom,
                                                                   u32 cap)
{
  const u32 start = min(c->levelStart[l], cap), cnt = min(c->levelCount[l], cap - start);
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
  {
    const u32 id = start + i;
    T mn[3], mx[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      mn[d] = Lim<T>::max();
      mx[d] = -Lim<T>::max();
    }
    const uint2 s = seg[id];
    for (u32 j = s.x; j < s.x + s.y; ++j)
    {
      const T* g = sortedGeom + u64(j) * 6;
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        mn[d] = smin(mn[d], g[d]);
        mx[d] = smax(mx[d], g[3 + d]);
      }
    }
    for (u32 ch = childBegin[id]; ch < childBegin[id + 1]; ++ch)
    {
      const T* g = geom + u64(ch) * 6;
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        mn[d] = smin(mn[d], g[d]);
        mx[d] = smax(mx[d], T(g[d] + g[3 + d])); // GetNodeBox: Max = minPoint + size
      }
    }
    T* o = geom + u64(id) * 6;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      o[d] = mn[d];
      o[3 + d] = mx[d] - mn[d];
    }
  }
}

template<typename T, typename K, bool IS_BOX>
int export_static_impl(TreeState& t, otg_static_layout* out, cudaStream_t st)
{
  const u64 mDyn = t.nodeCount;
  const u32 W = IS_BOX ? 6u : 3u;
  cudaError_t e;
  if ((e = t.stOrder.ensure(sizeof(u32) * mDyn)) || (e = t.stChildBegin.ensure(sizeof(u32) * (mDyn + 1))) ||
      (e = t.stSeg.ensure(sizeof(uint2) * mDyn)) || (e = t.stDepth.ensure(mDyn)) || (e = t.stGeom.ensure(sizeof(T) * W * mDyn)) ||
      (e = t.stCtl.ensure(sizeof(StaticCtl))))
    return cuda_status(e, "allocating the static layout");
  auto* ctl = t.stCtl.as<StaticCtl>();
  const K* keys = reinterpret_cast<const K*>(t.sortedKeys);
  static_init_kernel<<<1, 64, 0, st>>>(ctl, t.stOrder.as<u32>());
  for (u32 l = 0; l <= t.D; ++l)
  {
    static_count_kernel<<<kStaticBlocks, kStaticThreads, 0, st>>>(ctl, l, t.stOrder.as<u32>(), t.nodeLink.as<uint4>(), u32(mDyn));
    static_scan_kernel<<<1, 32, 0, st>>>(ctl, l, kStaticBlocks);
    static_assign_kernel<T, K, IS_BOX><<<kStaticBlocks, kStaticThreads, 0, st>>>(
      ctl, l, t.nodeLink.as<uint4>(), t.nodeDepth.as<unsigned char>(), keys, t.stOrder.as<u32>(), u32(mDyn), t.stChildBegin.as<u32>(),
      t.stSeg.as<uint2>(), t.stDepth.as<unsigned char>(), IS_BOX ? nullptr : t.stGeom.as<T>(), t.minTab.as<T>(), t.D, t.maxElem);
  }
  static_finish_kernel<<<1, 32, 0, st>>>(ctl, t.stChildBegin.as<u32>(), u32(mDyn));
  if constexpr (IS_BOX)
    for (u32 l = t.D + 1; l-- > 0;)
      static_mbr_kernel<T><<<kStaticBlocks, kStaticThreads, 0, st>>>(ctl, l, t.stChildBegin.as<u32>(), t.stSeg.as<uint2>(), t.sortedGeom.as<T>(),
                                                                   t.stGeom.as<T>(), u32(mDyn));
  StaticCtl h;
  e = cudaGetLastError();
  if (!e)
    e = cudaMemcpyAsync(&h, ctl, sizeof(StaticCtl), cudaMemcpyDeviceToHost, st);
  if (!e)
    e = cudaStreamSynchronize(st);
  if (e)
    return cuda_status(e, "computing the static layout");
  if (h.err)
  {
    set_error("static layout: inconsistent node links");
    return OTG_ERR_CUDA;
  }
  if (h.levelCount[t.D + 1] != 0)
  {
    set_error("static layout: more levels than the max depth allows");
    return OTG_ERR_CUDA;
  }
  if (h.covered != t.n)
  {
    set_error("static layout: some entity locations lie outside the grid (in no node of the tree)");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  const u64 m = h.levelStart[t.D + 1];
  out->node_count = m;
  out->child_begin_count = h.lastParentPlus1 ? u64(h.lastParentPlus1) + 1 : 1;
  out->entity_count = t.n;
  out->geometry_per_node = W;
  out->scalar_bytes = sizeof(T);
  out->child_begins = t.stChildBegin.as<u32>();
  out->entity_segments = t.stSeg.as<u32>();
  out->depth_ids = t.stDepth.as<uint8_t>();
  out->entity_storage = t.sortedIds.as<u32>();
  out->geometry = t.stGeom.p;
  return OTG_OK;
}

} // namespace

int export_static(TreeState& t, otg_static_layout* out, cudaStream_t st)
{
  if (!out)
  {
    set_error("otg_tree_export_static: null output");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  *out = otg_static_layout{};
  const bool box = t.kind != OTG_KIND_POINTS;
  out->geometry_per_node = box ? 6 : 3;
  out->scalar_bytes = t.scalar == OTG_SCALAR_F64 ? 8 : 4;
  if (!t.built)
  {
    set_error("otg_tree_export_static: the tree is not built");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (t.trees)
  {
    set_error("otg_tree_export_static: the static layout is defined for a single tree, not a forest");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (t.inserted)
  {
    // the reference's static tree has no Insert, and its layout is a Create's (one child segment per
    // node, entities only in leaves)
    set_error("otg_tree_export_static: the tree was changed by Insert; create it from all its entities instead");
    return OTG_ERR_NOT_SUPPORTED;
  }
  int rc = finish_build(t, st);
  if (rc)
    return rc;
  if (t.n == 0)
    return OTG_OK; // Create of no entities makes no node (core/ot_static_linear_core.h:539-540)
  if (!box)
  {
    // a point outside the space has the root's location and sorts first (key 0)
    u64 first = 0;
    cudaError_t e = cudaMemcpyAsync(&first, t.sortedKeys, t.keys32 ? 4 : 8, cudaMemcpyDeviceToHost, st);
    if (!e)
      e = cudaStreamSynchronize(st);
    if (e)
      return cuda_status(e, "reading the first location");
    if (first == 0)
    {
      set_error("otg_tree_export_static: the tree holds points outside its space, on which the reference's static build does not end");
      return OTG_ERR_INVALID_ARGUMENT;
    }
  }
  if (t.scalar == OTG_SCALAR_F64)
  {
    if (box)
      return t.keys32 ? export_static_impl<double, u32, true>(t, out, st) : export_static_impl<double, u64, true>(t, out, st);
    return t.keys32 ? export_static_impl<double, u32, false>(t, out, st) : export_static_impl<double, u64, false>(t, out, st);
  }
  if (box)
    return t.keys32 ? export_static_impl<float, u32, true>(t, out, st) : export_static_impl<float, u64, true>(t, out, st);
  return t.keys32 ? export_static_impl<float, u32, false>(t, out, st) : export_static_impl<float, u64, false>(t, out, st);
}

} // namespace otg
