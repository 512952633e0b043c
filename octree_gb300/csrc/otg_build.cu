// otg_build.cu — GPU Create of the Morton location-code tree.
//
// Replaces DynamicHashOrthoTreeCore::Create (core/ot_dynamic_hash_core.h:751-809):
//   1. space box: given, or the entities' bounding box (IGM::GetBoundingBoxAD,
//      detail/internal_geometry_module.h:342-370)                       -> bbox_kernel
//   2. grid factors and MinPoint node sizes (detail/si_grid.h:65-103,
//      core/ot_base.h:121-134)                                             -> space_setup_kernel
//   3. one location key per entity (si_mortongrid.h:69-97) fused with the radix digit
//      histograms of the sort                                              -> codegen_*_kernel
//   4. stable radix sort of (key, id) (replaces std::sort(par), :791-796)  -> otg_sort.cuh
//   5. entities gathered into tree order                                   -> gather_kernel
//   6. node emission, one launch per depth (BuildSubtree/ProcessNode,
//      :647-747): a node whose subtree holds more than maxElem entities and
//      d < maxDepth keeps its "stuck" entities (location depth == d) and
//      splits the rest into its <= 8 non-empty child key ranges            -> emit_level_kernel
//   7. MBR node boxes bottom-up (:1425-1450) for box trees, or the root box
//      widening of MinPoint trees built with a given box (:1573-1601)       -> mbr_level_kernel / root_box_kernel
//
// Key encoding (all keys sort exactly like the reference's compact Location (loc << 5 | depth),
// si_morton.h:117-143):
//   points: key = loc + 1, and 0 for entities outside a given box (Location(0, 0), which the
//           reference stores in the root, si_mortongrid.h:57-62). 3*D + 1 bits.
//   boxes : key = loc << 5 | depth. 3*D + 5 bits.
#include "otg_internal.h"
#include "otg_sort.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace otg
{

template<typename T>
struct OrderedBits;
template<>
struct OrderedBits<double>
{
  using type = unsigned long long;
};
template<>
struct OrderedBits<float>
{
  using type = unsigned int;
};

// ---------------------------------------------------------------- 1. bounding box
template<typename T, int W>
__global__ void __launch_bounds__(256) bbox_kernel(const T* __restrict__ ent, u64 n, typename OrderedBits<T>::type* acc)
{
  using B = typename OrderedBits<T>::type;
  B mn[3], mx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    mn[d] = B(~B(0));
    mx[d] = B(0);
  }
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    const T* e = ent + i * W;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      B lo = ordered_bits(e[d]);
      B hi = ordered_bits(e[W == 6 ? 3 + d : d]);
      mn[d] = lo < mn[d] ? lo : mn[d];
      mx[d] = hi > mx[d] ? hi : mx[d];
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      B a = __shfl_xor_sync(0xffffffffu, mn[d], o);
      B b = __shfl_xor_sync(0xffffffffu, mx[d], o);
      mn[d] = a < mn[d] ? a : mn[d];
      mx[d] = b > mx[d] ? b : mx[d];
    }
  }
  if ((threadIdx.x & 31) == 0)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      atomicMin(&acc[d], mn[d]);
      atomicMax(&acc[3 + d], mx[d]);
    }
  }
}

template<typename T>
__global__ void bbox_init_kernel(typename OrderedBits<T>::type* acc)
{
  using B = typename OrderedBits<T>::type;
  int d = threadIdx.x;
  if (d < 3)
  {
    acc[d] = B(~B(0));
    acc[3 + d] = B(0);
  }
}

// ---------------------------------------------------------------- 2. space
// si_grid.h:65-103 (factors), ot_base.h:121-134 (MinPoint node size table)
template<typename T>
__global__ void space_setup_kernel(Space<T>* sp, const typename OrderedBits<T>::type* acc, const T* box, u32 D, int isPoints)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  Space<T> s;
  for (int d = 0; d < 3; ++d)
  {
    if (box)
    {
      s.min[d] = box[d];
      s.max[d] = box[3 + d];
    }
    else
    {
      s.min[d] = from_ordered_bits(acc[d]);
      s.max[d] = from_ordered_bits(acc[3 + d]);
    }
    s.size[d] = s.max[d] - s.min[d];
  }
  s.D = D;
  const u64 res = u64(1) << D;
  const double subD = double(res);
  const float subF = float(res);
  for (int d = 0; d < 3; ++d)
  {
    s.rsizeD[d] = double(s.size[d]);
    s.derastD[d] = s.rsizeD[d] / subD;
    s.rastD[d] = s.rsizeD[d] == 0 ? 1.0 : (subD / s.rsizeD[d]);
    s.rsizeF[d] = float(s.size[d]);
    s.derastF[d] = s.rsizeF[d] / subF;
    s.rastF[d] = s.rsizeF[d] == 0 ? 1.0f : (subF / s.rsizeF[d]);
  }
  s.rasterDouble = (sizeof(T) == 8 || D >= 16) ? 1u : 0u;
  if (isPoints)
  {
    T lf = T(1.0);
    for (u32 d = 0; d < D + 2 && d < 22; ++d, lf *= T(0.5))
      for (int c = 0; c < 3; ++c)
        s.nodeSize[d][c] = s.size[c] * lf;
  }
  *sp = s;
}

// ---------------------------------------------------------------- 3. location keys
template<typename R, typename T>
struct Raster;
template<typename T>
struct Raster<double, T>
{
  static __device__ __forceinline__ double rsize(const Space<T>& s, int d) { return s.rsizeD[d]; }
  static __device__ __forceinline__ double rast(const Space<T>& s, int d) { return s.rastD[d]; }
  static __device__ __forceinline__ double derast(const Space<T>& s, int d) { return s.derastD[d]; }
};
template<typename T>
struct Raster<float, T>
{
  static __device__ __forceinline__ float rsize(const Space<T>& s, int d) { return s.rsizeF[d]; }
  static __device__ __forceinline__ float rast(const Space<T>& s, int d) { return s.rastF[d]; }
  static __device__ __forceinline__ float derast(const Space<T>& s, int d) { return s.derastF[d]; }
};

__device__ __forceinline__ u32 to_grid(double v) { return u32(v); } // C++ truncation
__device__ __forceinline__ u32 to_grid(float v) { return u32(v); }

// si_grid.h:145-175 GetPointGridID + si_morton.h Encode -> key (loc + 1, or 0 when outside)
template<typename T, typename R>
__device__ __forceinline__ u64 point_key(const T* p, const Space<T>& s, u32 maxRasterID)
{
  const T tol = base_tol<T>();
  u32 g[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    T pc = T(p[d]) - s.min[d];
    R rs = Raster<R, T>::rsize(s, d);
    if (pc < -tol || pc > rs + R(tol))
      return 0;
    if (pc <= 0)
      g[d] = 0;
    else
    {
      u32 rid = to_grid(R(pc) * Raster<R, T>::rast(s, d));
      g[d] = rid < maxRasterID ? rid : maxRasterID;
    }
  }
  return encode3(g[0], g[1], g[2]) + 1;
}

// si_grid.h:221-285 GetLooseBoxGridData<2.0> + si_mortongrid.h:78-88 -> loc << 5 | depth
template<typename T, typename R>
__device__ __forceinline__ u64 loose_box_key(const T* b, const Space<T>& s, u32 D)
{
  const T tol = base_tol<T>();
  // DoesRangeContainBoxAD(space, box, tol), internal_geometry_module.h:214-225
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    T rmin = s.min[d], rmax = s.max[d];
    if (rmin - tol > b[d] || b[d] > rmax + tol)
      return 0;
    if (rmin - tol > b[3 + d] || b[3 + d] > rmax + tol)
      return 0;
  }
  u32 g[3];
  R maxRel = R(0);
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    T center = (b[d] + b[3 + d]) * T(0.5);
    T bsize = T(b[3 + d] - b[d]);
    g[d] = to_grid(R(center - s.min[d]) * Raster<R, T>::rast(s, d));
    maxRel = smax(maxRel, R(bsize) * Raster<R, T>::rast(s, d));
  }
  u32 maxRelGrid = to_grid(ceil(maxRel));
  u32 level = 0;
  if (maxRelGrid != 0)
    level = 32u - __clz(maxRelGrid - 1u); // std::bit_width
  const u32 shift = level * 3u;
  u64 loc = encode3(g[0], g[1], g[2]);
  loc = shift < 64 ? ((loc >> shift) << shift) : 0;
  const u64 depth = u64(u32(D - level));
  return (loc << 5) | depth;
}

template<typename T, typename R, typename K, bool IS_BOX>
__global__ void __launch_bounds__(256) codegen_kernel(const T* __restrict__ ent, u64 n, const Space<T>* __restrict__ spg, K* __restrict__ keys,
                                                      u32* __restrict__ hist, u32 passes)
{
  __shared__ u32 sh[8][kRadix];
  __shared__ Space<T> s;
  for (int i = threadIdx.x; i < 8 * kRadix; i += blockDim.x)
    (&sh[0][0])[i] = 0;
  if (threadIdx.x == 0)
    s = *spg;
  __syncthreads();
  const u32 D = s.D;
  const u32 maxRasterID = (1u << D) - 1u;
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    u64 key;
    if constexpr (IS_BOX)
      key = loose_box_key<T, R>(ent + i * 6, s, D);
    else
      key = point_key<T, R>(ent + i * 3, s, maxRasterID);
    K k = K(key);
    keys[i] = k;
    for (u32 p = 0; p < passes; ++p)
      atomicAdd(&sh[p][(k >> (kRadixBits * p)) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  for (u32 p = 0; p < passes; ++p)
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
      if (sh[p][d])
        atomicAdd(&hist[p * kRadix + d], sh[p][d]);
}

// per-entity location keys in input order, reference layout (loc << 5 | depth)
template<typename T, typename R, bool IS_BOX>
__global__ void location_export_kernel(const T* __restrict__ ent, u64 n, const Space<T>* __restrict__ spg, u64* __restrict__ out)
{
  const Space<T> s = *spg;
  const u32 D = s.D;
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    if constexpr (IS_BOX)
      out[i] = loose_box_key<T, R>(ent + i * 6, s, D);
    else
    {
      u64 k = point_key<T, R>(ent + i * 3, s, (1u << D) - 1u);
      out[i] = k == 0 ? 0 : (((k - 1) << 5) | D);
    }
  }
}

// ---------------------------------------------------------------- 5. gather into tree order
template<typename T, int W>
__global__ void __launch_bounds__(256) gather_kernel(const T* __restrict__ ent, const u32* __restrict__ ids, u64 n, T* __restrict__ out)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    const u32 id = ids[i];
    if (id >= n)
      continue; // only reachable after a reported sort failure
    const T* src = ent + u64(id) * W;
    T* dst = out + i * W;
#pragma unroll
    for (int c = 0; c < W; ++c)
      dst[c] = src[c];
  }
}

// ---------------------------------------------------------------- 6. node emission
template<typename K>
__device__ __forceinline__ u32 lower_bound_key(const K* keys, u32 lo, u32 hi, u64 target)
{
  while (lo < hi)
  {
    u32 mid = lo + ((hi - lo) >> 1);
    if (u64(keys[mid]) < target)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}
template<typename K>
__device__ __forceinline__ u32 upper_bound_key(const K* keys, u32 lo, u32 hi, u64 target)
{
  while (lo < hi)
  {
    u32 mid = lo + ((hi - lo) >> 1);
    if (u64(keys[mid]) <= target)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// every third bit (inverse of part1by2)
__device__ __forceinline__ u32 compact1by2(u64 x)
{
  x &= 0x9249249249249249ULL;
  x = (x ^ (x >> 2)) & 0x30c30c30c30c30c3ULL;
  x = (x ^ (x >> 4)) & 0xf00f00f00f00f00fULL;
  x = (x ^ (x >> 8)) & 0x00ff0000ff0000ffULL;
  x = (x ^ (x >> 16)) & 0xffff00000000ffffULL;
  x = (x ^ (x >> 32)) & 0x00000000001fffffULL;
  return u32(x);
}

// MinPoint of a node: CalculateGridCellCenter(Decode(key), D - depth) - nodeSize[depth + 1]
// (si_grid.h:124-143, si_morton.h:576-622, ot_dynamic_hash_core.h:563-572)
template<typename T, typename R>
__device__ __forceinline__ void node_min_point(u64 key, u32 depth, const Space<T>& s, T out[3])
{
  const u32 D = s.D;
  const u64 loc = key ^ (u64(1) << (3 * depth));
  const u32 lvl = D - depth;
  const R halfGrid = R(u64(1) << lvl) * R(0.5);
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    u32 g = compact1by2(loc >> d) << lvl;
    T c = T((R(g) + halfGrid) * Raster<R, T>::derast(s, d)) + s.min[d];
    out[d] = c - s.nodeSize[depth + 1][d];
  }
}

template<typename T>
__global__ void root_init_kernel(uint4* link, u64* nodeKey, unsigned char* nodeDepth, u32* levelCount, u32 n)
{
  if (threadIdx.x == 0 && blockIdx.x == 0)
  {
    link[0] = make_uint4(0, 0, 0, n);
    nodeKey[0] = 1;
    nodeDepth[0] = 0;
    levelCount[0] = 1;
  }
}

__device__ __forceinline__ void level_range(const u32* levelCount, u32 d, u32& begin, u32& cnt)
{
  u32 b = 0;
  for (u32 j = 0; j < d; ++j)
    b += levelCount[j];
  begin = b;
  cnt = levelCount[d];
}

template<typename T, typename K, bool IS_BOX>
__global__ void __launch_bounds__(256) emit_level_kernel(u32 d, u64 maxElem, const K* __restrict__ keys, uint4* __restrict__ link,
                                                         u64* __restrict__ nodeKey, T* __restrict__ nodeBox, unsigned char* __restrict__ nodeDepth,
                                                         u32* __restrict__ levelCount, const Space<T>* __restrict__ spg, u64 maxNodes,
                                                         u32* __restrict__ err, u32* __restrict__ ownerNode, u32* __restrict__ nodeParent)
{
  __shared__ Space<T> s;
  if (threadIdx.x == 0)
    s = *spg;
  __syncthreads();
  const u32 D = s.D;
  u32 begin, cnt;
  level_range(levelCount, d, begin, cnt);
  const u32 childBase = begin + cnt;
  const int lane = threadIdx.x & 31;
  for (u32 i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < cnt; i0 += gridDim.x * blockDim.x)
  {
    const u32 i = i0 + lane;
    const bool active = i < cnt;
    const u32 node = begin + i;
    u32 bounds[9];
    u32 nchild = 0;
    u32 b = 0, e = 0, ownEnd = 0;
    u64 key = 1;
    if (active)
    {
      uint4 L = link[node];
      key = nodeKey[node];
      b = L.y;
      e = L.w;
      const u64 count = u64(e - b);
      const bool split = count > maxElem && d < D;
      u32 sEnd = b;
      const u64 lmin = (key ^ (u64(1) << (3 * d))) << (3 * (D - d));
      if (split)
      {
        if constexpr (IS_BOX)
          sEnd = upper_bound_key(keys, b, e, (lmin << 5) | u64(d)); // ProcessNode partition_point, :658-671
        else
          sEnd = (d == 0) ? upper_bound_key(keys, b, e, 0) : b;
      }
      ownEnd = split ? sEnd : e;
      if (split && sEnd < e)
      {
        const u64 S = u64(1) << (3 * (D - d - 1));
        bounds[0] = sEnd;
#pragma unroll
        for (int c = 1; c <= 8; ++c)
        {
          const u64 L0 = lmin + u64(c) * S;
          const u64 target = IS_BOX ? (L0 << 5) : (L0 + 1);
          bounds[c] = lower_bound_key(keys, bounds[c - 1], e, target);
        }
#pragma unroll
        for (int c = 0; c < 8; ++c)
          nchild += bounds[c + 1] > bounds[c] ? 1u : 0u;
      }
    }
    // warp-aggregated allocation of the children slots (children of one node are contiguous)
    u32 incl = nchild;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      u32 y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o)
        incl += y;
    }
    u32 warpTotal = __shfl_sync(0xffffffffu, incl, 31);
    u32 warpBase = 0;
    if (lane == 31 && warpTotal)
      warpBase = atomicAdd(&levelCount[d + 1], warpTotal);
    warpBase = __shfl_sync(0xffffffffu, warpBase, 31);
    const u32 firstChild = childBase + warpBase + incl - nchild;
    if (active)
    {
      if (u64(firstChild) + nchild > maxNodes)
      {
        atomicOr(err, kErrCapacity);
        nchild = 0;
      }
      u32 j = 0;
      for (int c = 0; c < 8 && nchild; ++c)
      {
        if (bounds[c + 1] > bounds[c])
        {
          const u32 ci = firstChild + j++;
          nodeKey[ci] = (key << 3) | u64(c);
          link[ci] = make_uint4(0, bounds[c], bounds[c], bounds[c + 1]);
          nodeDepth[ci] = (unsigned char)(d + 1);
          if (nodeParent)
            nodeParent[ci] = node;
        }
      }
      link[node] = make_uint4((nchild ? (firstChild & kFirstChildMask) : 0u) | (nchild << kChildShift), b, ownEnd, e);
      if (ownerNode)
        for (u32 q = b; q < ownEnd; ++q)
          ownerNode[q] = node;
      if constexpr (!IS_BOX)
      {
        T mn[3];
        if (s.rasterDouble)
          node_min_point<T, double>(key, d, s, mn);
        else
          node_min_point<T, float>(key, d, s, mn);
        T* nb = nodeBox + u64(node) * 6;
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
          nb[c] = mn[c];
          nb[3 + c] = s.nodeSize[d][c];
        }
      }
    }
  }
}

// ---------------------------------------------------------------- 7. node boxes
// ot_dynamic_hash_core.h:1425-1450 (children first, then own entities), one depth per launch
template<typename T>
__global__ void __launch_bounds__(256) mbr_level_kernel(u32 d, const u32* __restrict__ levelCount, const uint4* __restrict__ link,
                                                        const T* __restrict__ sortedGeom, T* __restrict__ nodeBox, T* __restrict__ nodeMax)
{
  u32 begin, cnt;
  level_range(levelCount, d, begin, cnt);
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
  {
    const u32 node = begin + i;
    const uint4 L = link[node];
    T mn[3], mx[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      mn[c] = Lim<T>::max();
      mx[c] = -Lim<T>::max();
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (L.z > L.w || (cc && fc <= node))
      continue; // malformed link: emission reports capacity errors separately
    for (u32 k = 0; k < cc; ++k)
    {
      const T* cb = nodeBox + u64(fc + k) * 6;
      const T* cm = nodeMax + u64(fc + k) * 3;
#pragma unroll
      for (int c = 0; c < 3; ++c)
      {
        mn[c] = smin(mn[c], cb[c]);
        mx[c] = smax(mx[c], cm[c]);
      }
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      const T* g = sortedGeom + u64(e) * 6;
#pragma unroll
      for (int c = 0; c < 3; ++c)
      {
        mn[c] = smin(mn[c], g[c]);
        mx[c] = smax(mx[c], g[3 + c]);
      }
    }
    T* nb = nodeBox + u64(node) * 6;
    T* nm = nodeMax + u64(node) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      nb[c] = mn[c];
      nb[3 + c] = mx[c] - mn[c];
      nm[c] = mx[c];
    }
  }
}

// ot_dynamic_hash_core.h:1573-1601 InitializeRootNodeBox (MinPoint, out-of-space insertion allowed):
// the root box becomes the union of its nominal box and its own entities.
template<typename T>
__global__ void __launch_bounds__(256) root_box_kernel(const uint4* __restrict__ link, const T* __restrict__ sortedGeom, T* __restrict__ nodeBox,
                                                       Space<T>* sp)
{
  __shared__ T smn[3][256], smx[3][256];
  const uint4 L = link[0];
  T mn[3], mx[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
  {
    mn[c] = Lim<T>::max();
    mx[c] = -Lim<T>::max();
  }
  for (u32 e = L.y + threadIdx.x; e < L.z; e += blockDim.x)
  {
    const T* p = sortedGeom + u64(e) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      mn[c] = smin(mn[c], p[c]);
      mx[c] = smax(mx[c], p[c]);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
  {
    smn[c][threadIdx.x] = mn[c];
    smx[c][threadIdx.x] = mx[c];
  }
  __syncthreads();
  if (threadIdx.x == 0)
  {
    T bmin[3], bmax[3];
    for (int c = 0; c < 3; ++c)
    {
      bmin[c] = nodeBox[c];
      bmax[c] = nodeBox[c] + nodeBox[3 + c];
    }
    for (int t = 0; t < blockDim.x; ++t)
      for (int c = 0; c < 3; ++c)
      {
        bmin[c] = smin(bmin[c], smn[c][t]);
        bmax[c] = smax(bmax[c], smx[c][t]);
      }
    for (int c = 0; c < 3; ++c)
    {
      nodeBox[c] = bmin[c];
      nodeBox[3 + c] = bmax[c] - bmin[c];
      sp->nodeSize[0][c] = nodeBox[3 + c];
    }
  }
}

// ---------------------------------------------------------------- host orchestration
static int grid_blocks(u64 n, int perBlock = 256, int maxBlocks = 152 * 16)
{
  u64 b = (n + perBlock - 1) / perBlock;
  return int(std::max<u64>(1, std::min<u64>(b, u64(maxBlocks))));
}

// detail/utils.h:613-622 EstimateMaxDepth (3-D)
static u32 estimate_max_depth(u64 n, u64 maxElem)
{
  if (n <= maxElem)
    return 2;
  u64 nLeaf = n / maxElem;
  u32 d = u32(std::log2(double(nLeaf)) / 3.0);
  return std::clamp<u32>(d, 2u, 21u);
}

template<typename T, typename K, bool IS_BOX>
static int build_impl(TreeState& t, const void* box, u64 n, cudaStream_t st)
{
  constexpr int W = IS_BOX ? 6 : 3;
  using B = typename OrderedBits<T>::type;
  const u32 D = t.D;
  const u32 bits = IS_BOX ? 3 * D + 5 : 3 * D + 1;
  const u32 passes = (bits + kRadixBits - 1) / kRadixBits;
  cudaError_t e;

  // buffers
  const u64 maxNodes = n + u64(D) * (n / (t.maxElem + 1) + 1) + 2;
  t.maxNodes = maxNodes;
  if ((e = t.keysA.ensure(sizeof(K) * n)) || (e = t.keysB.ensure(sizeof(K) * n)) || (e = t.sortedIds.ensure(sizeof(u32) * n)) ||
      (e = t.valsB.ensure(sizeof(u32) * n)) || (e = t.sortedGeom.ensure(sizeof(T) * W * n)) || (e = t.nodeLink.ensure(sizeof(uint4) * maxNodes)) ||
      (e = t.nodeKey.ensure(sizeof(u64) * maxNodes)) || (e = t.nodeBox.ensure(sizeof(T) * 6 * maxNodes)) ||
      (e = t.nodeDepth.ensure(maxNodes)) || (e = t.levelCount.ensure(sizeof(u32) * 32)) || (e = t.space.ensure(sizeof(Space<T>))) ||
      (e = t.sortScratch.ensure(SortScratch::bytes(n, passes))) || (e = t.bboxBits.ensure(sizeof(B) * 6)) ||
      (IS_BOX && ((e = t.nodeMax.ensure(sizeof(T) * 3 * maxNodes)) || (e = t.ownerNode.ensure(sizeof(u32) * n)) ||
                  (e = t.nodeParent.ensure(sizeof(u32) * maxNodes)))))
    return cuda_status(e, "allocating tree buffers");

  Profiler& prof = profiler();
  prof.reset();
  prof.mark("setup", st);
  SortScratch ss;
  ss.carve(t.sortScratch.p, n, passes);
  cudaMemsetAsync(t.sortScratch.p, 0, SortScratch::bytes(n, passes), st);
  cudaMemsetAsync(t.levelCount.p, 0, sizeof(u32) * 32, st);

  const T* ent = t.entities.as<T>();
  Space<T>* sp = t.space.as<Space<T>>();
  if (!box)
  {
    prof.mark("bbox", st);
    bbox_init_kernel<T><<<1, 32, 0, st>>>(t.bboxBits.as<B>());
    bbox_kernel<T, W><<<grid_blocks(n, 256, 152 * 8), 256, 0, st>>>(ent, n, t.bboxBits.as<B>());
  }
  space_setup_kernel<T><<<1, 1, 0, st>>>(sp, t.bboxBits.as<B>(), (const T*)box, D, IS_BOX ? 0 : 1);

  const bool rasterDouble = (sizeof(T) == 8) || D >= 16;
  prof.mark("codegen", st);
  if (rasterDouble)
    codegen_kernel<T, double, K, IS_BOX><<<grid_blocks(n, 256, 152 * 8), 256, 0, st>>>(ent, n, sp, t.keysA.as<K>(), ss.hist, passes);
  else
    codegen_kernel<T, float, K, IS_BOX><<<grid_blocks(n, 256, 152 * 8), 256, 0, st>>>(ent, n, sp, t.keysA.as<K>(), ss.hist, passes);

  prof.mark("sort", st);
  bool inB = onesweep_passes<K>(t.keysA.as<K>(), t.sortedIds.as<u32>(), t.keysB.as<K>(), t.valsB.as<u32>(), n, 0, passes, true, ss, t.err.as<u32>(), st);
  if (inB)
  {
    std::swap(t.sortedIds, t.valsB);
    t.sortedKeys = t.keysB.p;
  }
  else
    t.sortedKeys = t.keysA.p;
  const K* keys = reinterpret_cast<const K*>(t.sortedKeys);

  prof.mark("gather", st);
  gather_kernel<T, W><<<grid_blocks(n, 256, 152 * 8), 256, 0, st>>>(ent, t.sortedIds.as<u32>(), n, t.sortedGeom.as<T>());

  prof.mark("emit", st);
  root_init_kernel<T><<<1, 32, 0, st>>>(t.nodeLink.as<uint4>(), t.nodeKey.as<u64>(), t.nodeDepth.as<unsigned char>(), t.levelCount.as<u32>(), u32(n));
  const int emitBlocks = grid_blocks(n / std::max<u64>(1, t.maxElem / 2), 256, 152 * 4);
  for (u32 d = 0; d <= D; ++d)
    emit_level_kernel<T, K, IS_BOX><<<emitBlocks, 256, 0, st>>>(d, t.maxElem, keys, t.nodeLink.as<uint4>(), t.nodeKey.as<u64>(), t.nodeBox.as<T>(),
                                                                t.nodeDepth.as<unsigned char>(), t.levelCount.as<u32>(), sp, maxNodes, t.err.as<u32>(),
                                                                IS_BOX ? t.ownerNode.as<u32>() : nullptr, IS_BOX ? t.nodeParent.as<u32>() : nullptr);
  prof.mark("geometry", st);
  if constexpr (IS_BOX)
  {
    for (int d = int(D); d >= 0; --d)
      mbr_level_kernel<T><<<emitBlocks, 256, 0, st>>>(u32(d), t.levelCount.as<u32>(), t.nodeLink.as<uint4>(), t.sortedGeom.as<T>(), t.nodeBox.as<T>(),
                                                      t.nodeMax.as<T>());
  }
  else
  {
    if (box)
      root_box_kernel<T><<<1, 256, 0, st>>>(t.nodeLink.as<uint4>(), t.sortedGeom.as<T>(), t.nodeBox.as<T>(), sp);
  }
  prof.mark("end", st);
  return cuda_status(cudaGetLastError(), "launching build kernels");
}

int build_tree(TreeState& t, const void* entities, u64 n, u32 maxDepth, const void* box, u64 maxElem, int mem, cudaStream_t st)
{
  const bool isBox = t.kind == OTG_KIND_BOXES;
  const int W = isBox ? 6 : 3;
  const size_t esz = t.scalar == OTG_SCALAR_F64 ? 8 : 4;
  if (maxElem == 0)
  {
    set_error("maxElementNo must be larger than 0");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (n >= (u64(1) << 30))
  {
    set_error("entity count must be below 2^30");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  const u32 D = (maxDepth == 0) ? estimate_max_depth(n, maxElem) : maxDepth;
  // core/ot_base.h:104-108 plus the compact Location limit of 19 levels (si_morton.h:149)
  if (D < 1 || D > 19)
  {
    set_error("maxDepthID must be in [1, 19]");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  t.n = n;
  t.D = D;
  t.maxElem = maxElem;
  t.built = false;
  t.countsKnown = false;
  t.boxGiven = box != nullptr;
  cudaError_t e;
  if ((e = t.entities.ensure(esz * W * n)) || (e = t.err.ensure(sizeof(u32) * 4)))
    return cuda_status(e, "allocating entity buffer");
  cudaMemsetAsync(t.err.p, 0, sizeof(u32) * 4, st);
  if (n)
  {
    e = cudaMemcpyAsync(t.entities.p, entities, esz * W * n, mem == OTG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st);
    if (e)
      return cuda_status(e, "copying entities");
  }
  // the box is read by a kernel: stage it in device memory
  DevBuf& boxBuf = t.boxDev;
  const void* dbox = nullptr;
  if (box)
  {
    if ((e = boxBuf.ensure(esz * 6)))
      return cuda_status(e, "allocating box");
    if ((e = cudaMemcpyAsync(boxBuf.p, box, esz * 6, mem == OTG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st)))
      return cuda_status(e, "copying box");
    dbox = boxBuf.p;
  }
  if (n == 0)
  {
    t.built = true;
    t.nodeCount = 1;
    t.countsKnown = true;
    t.levelCountsHost.assign(1, 1);
    if (mem == OTG_MEM_HOST)
      cudaStreamSynchronize(st);
    return OTG_OK;
  }
  const u32 bits = isBox ? 3 * D + 5 : 3 * D + 1;
  t.keys32 = bits <= 32;
  // node links pack the first-child index in 28 bits
  if (n + u64(D) * (n / (maxElem + 1) + 1) + 2 >= (u64(1) << kChildShift))
  {
    set_error("entity count too large for the 28-bit node index of this build");
    return OTG_ERR_NOT_SUPPORTED;
  }
  int rc;
  if (t.scalar == OTG_SCALAR_F64)
  {
    if (isBox)
      rc = t.keys32 ? build_impl<double, u32, true>(t, dbox, n, st) : build_impl<double, u64, true>(t, dbox, n, st);
    else
      rc = t.keys32 ? build_impl<double, u32, false>(t, dbox, n, st) : build_impl<double, u64, false>(t, dbox, n, st);
  }
  else
  {
    if (isBox)
      rc = t.keys32 ? build_impl<float, u32, true>(t, dbox, n, st) : build_impl<float, u64, true>(t, dbox, n, st);
    else
      rc = t.keys32 ? build_impl<float, u32, false>(t, dbox, n, st) : build_impl<float, u64, false>(t, dbox, n, st);
  }
  if (rc)
    return rc;
  t.built = true;
  if (mem == OTG_MEM_HOST)
    return finish_build(t, st);
  return OTG_OK;
}

int finish_build(TreeState& t, cudaStream_t st)
{
  if (t.countsKnown)
    return OTG_OK;
  u32 hostErr = 0;
  std::vector<u32> lc(32, 0);
  cudaError_t e = cudaMemcpyAsync(&hostErr, t.err.p, sizeof(u32), cudaMemcpyDeviceToHost, st);
  if (!e && t.n)
    e = cudaMemcpyAsync(lc.data(), t.levelCount.p, sizeof(u32) * 32, cudaMemcpyDeviceToHost, st);
  if (!e)
    e = cudaStreamSynchronize(st);
  if (e)
    return cuda_status(e, "finishing build");
  if (hostErr & kErrTimeout)
  {
    set_error("radix sort look-back wait ran out of its iteration limit");
    return OTG_ERR_TIMEOUT;
  }
  if (hostErr & kErrCapacity)
  {
    set_error("node capacity exceeded during emission");
    return OTG_ERR_OUT_OF_MEMORY;
  }
  if (t.n)
  {
    t.levelCountsHost.assign(lc.begin(), lc.begin() + t.D + 1);
    u64 s = 0;
    for (u32 v : t.levelCountsHost)
      s += v;
    t.nodeCount = s;
  }
  t.countsKnown = true;
  return OTG_OK;
}

int export_locations(const TreeState& t, u64* keys, int mem, cudaStream_t st)
{
  if (t.n == 0)
    return OTG_OK;
  DevBuf tmp;
  u64* out = keys;
  if (mem == OTG_MEM_HOST)
  {
    if (cudaError_t e = tmp.ensure(sizeof(u64) * t.n))
      return cuda_status(e, "allocating export buffer");
    out = tmp.as<u64>();
  }
  const bool isBox = t.kind == OTG_KIND_BOXES;
  const bool rd = t.scalar == OTG_SCALAR_F64 || t.D >= 16;
  const int blocks = grid_blocks(t.n);
  if (t.scalar == OTG_SCALAR_F64)
  {
    auto sp = t.space.as<Space<double>>();
    if (isBox)
      location_export_kernel<double, double, true><<<blocks, 256, 0, st>>>(t.entities.as<double>(), t.n, sp, out);
    else
      location_export_kernel<double, double, false><<<blocks, 256, 0, st>>>(t.entities.as<double>(), t.n, sp, out);
  }
  else
  {
    auto sp = t.space.as<Space<float>>();
    if (isBox)
    {
      if (rd)
        location_export_kernel<float, double, true><<<blocks, 256, 0, st>>>(t.entities.as<float>(), t.n, sp, out);
      else
        location_export_kernel<float, float, true><<<blocks, 256, 0, st>>>(t.entities.as<float>(), t.n, sp, out);
    }
    else
    {
      if (rd)
        location_export_kernel<float, double, false><<<blocks, 256, 0, st>>>(t.entities.as<float>(), t.n, sp, out);
      else
        location_export_kernel<float, float, false><<<blocks, 256, 0, st>>>(t.entities.as<float>(), t.n, sp, out);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (!e && mem == OTG_MEM_HOST)
  {
    e = cudaMemcpyAsync(keys, out, sizeof(u64) * t.n, cudaMemcpyDeviceToHost, st);
    if (!e)
      e = cudaStreamSynchronize(st);
  }
  tmp.release();
  return cuda_status(e, "exporting locations");
}

int export_nodes(const TreeState& t, u64* keys, double* minSize, u64* eoff, u32* eids, u32* childCount)
{
  const u64 m = t.nodeCount;
  std::vector<uint4> link(m);
  std::vector<u32> ids(t.n);
  cudaError_t e = cudaSuccess;
  if (t.n == 0)
  {
    keys[0] = 1;
    for (int c = 0; c < 6; ++c)
      minSize[c] = 0;
    eoff[0] = eoff[1] = 0;
    if (childCount)
      childCount[0] = 0;
    return OTG_OK;
  }
  e = cudaMemcpy(link.data(), t.nodeLink.p, sizeof(uint4) * m, cudaMemcpyDeviceToHost);
  if (!e)
    e = cudaMemcpy(keys, t.nodeKey.p, sizeof(u64) * m, cudaMemcpyDeviceToHost);
  if (!e)
    e = cudaMemcpy(ids.data(), t.sortedIds.p, sizeof(u32) * t.n, cudaMemcpyDeviceToHost);
  if (!e)
  {
    if (t.scalar == OTG_SCALAR_F64)
      e = cudaMemcpy(minSize, t.nodeBox.p, sizeof(double) * 6 * m, cudaMemcpyDeviceToHost);
    else
    {
      std::vector<float> f(6 * m);
      e = cudaMemcpy(f.data(), t.nodeBox.p, sizeof(float) * 6 * m, cudaMemcpyDeviceToHost);
      for (u64 i = 0; i < 6 * m; ++i)
        minSize[i] = f[i];
    }
  }
  if (e)
    return cuda_status(e, "exporting nodes");
  u64 off = 0;
  for (u64 i = 0; i < m; ++i)
  {
    eoff[i] = off;
    for (u32 j = link[i].y; j < link[i].z; ++j)
      eids[off++] = ids[j];
    if (childCount)
      childCount[i] = link[i].x >> kChildShift;
  }
  eoff[m] = off;
  return OTG_OK;
}

} // namespace otg
