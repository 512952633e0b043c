// otg_build.cu — GPU Create of the Morton location-code tree.
//
// Replaces DynamicHashOrthoTreeCore::Create (core/ot_dynamic_hash_core.h:751-809):
//   1. space box: given, or the entities' bounding box (IGM::GetBoundingBoxAD,
//      detail/internal_geometry_module.h:342-370)                       -> bbox_kernel
//   2. grid factors and MinPoint node sizes (detail/si_grid.h:65-103,
//      core/ot_base.h:121-134), exact rasterisation thresholds and the
//      MinPoint node table (otg_raster.cuh)                              -> space_setup / raster_tables / node_min_table
//   3. one location key per entity (si_mortongrid.h:69-97) fused with the radix digit
//      histograms of the sort; a point coordinate's cell from its FP32 estimate where that clears
//      the estimate's rounding margin, else integer compares against the thresholds -> codegen_kernel
//   4. stable radix sort of (key, id) (replaces std::sort(par), :791-796): digit bases
//      per pass, then one onesweep launch per 8-bit digit             -> digit_base / onesweep (otg_sort.cuh)
//   5. entities gathered into tree order                                   -> gather_kernel
//   6. node emission, one launch per depth (BuildSubtree/ProcessNode,
//      :647-747): a node whose subtree holds more than maxElem entities and
//      d < maxDepth keeps its "stuck" entities (location depth == d) and
//      splits the rest into its <= 8 non-empty child key ranges            -> emit_classify / emit_split
//   7. MBR node boxes bottom-up (:1425-1450) for box trees, or the root box
//      widening of MinPoint trees built with a given box (:1573-1601)       -> mbr_level_kernel / root_box_kernel
//
// Key encoding (all keys sort exactly like the reference's compact Location (loc << 5 | depth),
// si_morton.h:117-143):
//   points: key = loc + 1, and 0 for entities outside a given box (Location(0, 0), which the
//           reference stores in the root, si_mortongrid.h:57-62). 3*D + 1 bits.
//   boxes : key = loc << 5 | depth. 3*D + 5 bits.
#include "otg_internal.h"
#include "otg_raster.cuh"
#include "otg_sort.cuh"
#include "otg_sort_chunked.cuh"
#include "otg_query.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace otg
{

// entities handled per thread step: 48 bytes = three 16-byte vector loads
template<typename T, int W>
struct Chunk
{
  static constexpr int E = 48 / int(sizeof(T) * W);
  static_assert(E >= 1 && E * int(sizeof(T)) * W == 48, "chunk must be 48 bytes");
};

// loads entities [first, first + E) (clipped at n) into v; vector loads when aligned and whole.
// Every index is a compile-time constant after unrolling, so v stays in registers.
template<typename T, int W>
__device__ __forceinline__ int load_chunk(const T* __restrict__ ent, u64 n, u64 first, bool vec, T (&v)[Chunk<T, W>::E * W])
{
  constexpr int E = Chunk<T, W>::E;
  if (vec && first + E <= n)
  {
    // typed vector loads (no union: a union of vectors and scalars is kept in local memory)
    if constexpr (sizeof(T) == 8)
    {
      const double2* src = reinterpret_cast<const double2*>(ent + first * W);
#pragma unroll
      for (int j = 0; j < 3; ++j)
      {
        const double2 x = __ldg(src + j);
        v[2 * j] = x.x;
        v[2 * j + 1] = x.y;
      }
    }
    else
    {
      const float4* src = reinterpret_cast<const float4*>(ent + first * W);
#pragma unroll
      for (int j = 0; j < 3; ++j)
      {
        const float4 x = __ldg(src + j);
        v[4 * j] = x.x;
        v[4 * j + 1] = x.y;
        v[4 * j + 2] = x.z;
        v[4 * j + 3] = x.w;
      }
    }
    return E;
  }
  const int cnt = int(min(u64(E), n - first));
#pragma unroll
  for (int k = 0; k < E * W; ++k)
    v[k] = (k < cnt * W) ? ent[first * W + k] : T(0);
  return cnt;
}

// ---------------------------------------------------------------- 1. bounding box
template<typename T, int W>
__global__ void __launch_bounds__(256) bbox_kernel(const T* __restrict__ ent, u64 n, bool vec, typename Ord<T>::U* acc)
{
  using O = Ord<T>;
  using U = typename O::U;
  constexpr int E = Chunk<T, W>::E;
  U mn[3], mx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    mn[d] = U(~U(0));
    mx[d] = U(0);
  }
  const u64 chunks = (n + E - 1) / E;
  for (u64 c = blockIdx.x * u64(blockDim.x) + threadIdx.x; c < chunks; c += u64(gridDim.x) * blockDim.x)
  {
    T v[E * W];
    const int cnt = load_chunk<T, W>(ent, n, c * E, vec, v);
#pragma unroll
    for (int k = 0; k < E; ++k)
    {
      if (k >= cnt)
        break;
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        const U lo = ord_bits(v[k * W + d]);
        const U hi = W == 6 ? ord_bits(v[k * W + 3 + d]) : lo;
        mn[d] = lt_ord(lo, mn[d]) ? lo : mn[d];
        mx[d] = lt_ord(mx[d], hi) ? hi : mx[d];
      }
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      U a = __shfl_xor_sync(0xffffffffu, mn[d], o);
      U b = __shfl_xor_sync(0xffffffffu, mx[d], o);
      mn[d] = lt_ord(a, mn[d]) ? a : mn[d];
      mx[d] = lt_ord(mx[d], b) ? b : mx[d];
    }
  }
  // block reduction, then one atomic per block and coordinate (same-address atomics serialise)
  __shared__ U smn[3][8], smx[3][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      smn[d][warp] = mn[d];
      smx[d][warp] = mx[d];
    }
  __syncthreads();
  if (threadIdx.x < 3)
  {
    const int d = threadIdx.x;
    U a = smn[d][0], b = smx[d][0];
    for (int w = 1; w < int(blockDim.x >> 5); ++w)
    {
      a = smn[d][w] < a ? smn[d][w] : a;
      b = smx[d][w] > b ? smx[d][w] : b;
    }
    atomicMin(&acc[d], a);
    atomicMax(&acc[3 + d], b);
  }
}

// Upload and bounding box in one pass over host-mapped entities (16-byte aligned): consecutive
// threads read consecutive 16-byte units, so the reads over the host link are whole lines; every
// unit is written to the device copy, and each scalar updates the min or max of its dimension
// (point coordinates both; box minima the min, box maxima the max).
template<typename T, int W>
__global__ void __launch_bounds__(256) pull_bbox_kernel(const T* __restrict__ src, u64 n, T* __restrict__ dst, typename Ord<T>::U* acc)
{
  using U = typename Ord<T>::U;
  using V = typename std::conditional<sizeof(T) == 8, double2, float4>::type;
  constexpr int PER = int(16 / sizeof(T));
  U mn[3], mx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    mn[d] = U(~U(0));
    mx[d] = U(0);
  }
  auto take = [&](T val, u32 c) {
    const U o = ord_bits(val);
    const u32 d = c < 3 ? c : c - 3;
    const bool lo = W == 3 || c < 3, hi = W == 3 || c >= 3;
    if (d == 0)
    {
      mn[0] = lo && lt_ord(o, mn[0]) ? o : mn[0];
      mx[0] = hi && lt_ord(mx[0], o) ? o : mx[0];
    }
    else if (d == 1)
    {
      mn[1] = lo && lt_ord(o, mn[1]) ? o : mn[1];
      mx[1] = hi && lt_ord(mx[1], o) ? o : mx[1];
    }
    else
    {
      mn[2] = lo && lt_ord(o, mn[2]) ? o : mn[2];
      mx[2] = hi && lt_ord(mx[2], o) ? o : mx[2];
    }
  };
  const u64 total = n * W, units = total / PER;
  const u64 stride = u64(gridDim.x) * blockDim.x;
  for (u64 u = blockIdx.x * u64(blockDim.x) + threadIdx.x; u < units; u += stride)
  {
    const V x = reinterpret_cast<const V*>(src)[u];
    reinterpret_cast<V*>(dst)[u] = x;
    u32 c = u32((u * PER) % W);
    if constexpr (sizeof(T) == 8)
    {
      take(x.x, c);
      take(x.y, c + 1 == W ? 0 : c + 1);
    }
    else
    {
      take(x.x, c);
      c = c + 1 == W ? 0 : c + 1;
      take(x.y, c);
      c = c + 1 == W ? 0 : c + 1;
      take(x.z, c);
      c = c + 1 == W ? 0 : c + 1;
      take(x.w, c);
    }
  }
  for (u64 j = units * PER + blockIdx.x * u64(blockDim.x) + threadIdx.x; j < total; j += stride)
  {
    const T val = src[j];
    dst[j] = val;
    take(val, u32(j % W));
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      U a = __shfl_xor_sync(0xffffffffu, mn[d], o);
      U b = __shfl_xor_sync(0xffffffffu, mx[d], o);
      mn[d] = lt_ord(a, mn[d]) ? a : mn[d];
      mx[d] = lt_ord(mx[d], b) ? b : mx[d];
    }
  }
  __shared__ U smn[3][8], smx[3][8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      smn[d][warp] = mn[d];
      smx[d][warp] = mx[d];
    }
  __syncthreads();
  if (threadIdx.x < 3)
  {
    const int d = threadIdx.x;
    U a = smn[d][0], b = smx[d][0];
    for (int w = 1; w < int(blockDim.x >> 5); ++w)
    {
      a = smn[d][w] < a ? smn[d][w] : a;
      b = smx[d][w] > b ? smx[d][w] : b;
    }
    atomicMin(&acc[d], a);
    atomicMax(&acc[3 + d], b);
  }
}

template<typename U>
__global__ void bbox_init_kernel(U* acc)
{
  int d = threadIdx.x;
  if (d < 3)
  {
    acc[d] = U(~U(0));
    acc[3 + d] = U(0);
  }
}

// ---------------------------------------------------------------- 2. space
// si_grid.h:65-103 (factors), ot_base.h:121-134 (MinPoint node size table)
template<typename T>
__device__ void make_space(Space<T>& s, const typename Ord<T>::U* acc, const T* box, u32 D, int isPoints)
{
  for (int d = 0; d < 3; ++d)
  {
    if (box)
    {
      s.min[d] = box[d];
      s.max[d] = box[3 + d];
    }
    else
    {
      s.min[d] = Ord<T>::val(acc[d]);
      s.max[d] = Ord<T>::val(acc[3 + d]);
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
  for (u32 d = 0; d < 22; ++d)
    for (int c = 0; c < 3; ++c)
      s.nodeSize[d][c] = T(0);
  if (isPoints)
  {
    T lf = T(1.0);
    for (u32 d = 0; d < D + 2 && d < 22; ++d, lf *= T(0.5))
      for (int c = 0; c < 3; ++c)
        s.nodeSize[d][c] = s.size[c] * lf;
  }
}

template<typename T>
__global__ void space_setup_kernel(Space<T>* sp, const typename Ord<T>::U* acc, const T* box, u32 D, int isPoints)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  Space<T> s;
  make_space(s, acc, box, D, isPoints);
  *sp = s;
}

// ---------------------------------------------------------------- 3. location keys
// Reference formulas, one entity (used for exports; the build uses the threshold tables).
// si_grid.h:145-175 GetPointGridID + si_morton.h Encode -> key (loc + 1, or 0 when outside)
template<typename T, typename R>
__device__ __forceinline__ u64 point_key_ref(const T* p, const Space<T>& s, u32 maxRasterID)
{
  u32 g[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    if (point_below_ref<T, R>(p[d], s, d) || point_above_ref<T, R>(p[d], s, d))
      return 0;
    g[d] = point_cell_ref<T, R>(p[d], s, d, maxRasterID);
  }
  return encode3(g[0], g[1], g[2]) + 1;
}

// si_grid.h:177-219 GetBoxGridID + si_morton.h:698-722 GetRangeLocation (regular box trees, loose
// factor 1.0) -> loc << 5 | depth: the cells of the min and max corner (the max cell stepped back
// when it falls on a cell boundary or past the grid) and their lowest common ancestor. Outside
// the space: the root's location (key 0). The arithmetic is the reference's, operation by operation.
// A min corner in cell 2^D (a box on the max face of the space, within the tolerance) is where the
// reference asserts (si_grid.h:213); it returns kBadRegularBox, which the build reports.
constexpr u64 kBadRegularBox = ~u64(0);
template<typename T, typename R>
__device__ __forceinline__ u64 regular_box_key_ref(const T* b, const Space<T>& s, u32 D)
{
  const T tol = base_tol<T>();
  const u32 res = 1u << D;
  const R zero = R(0), maxR = R(res);
  u32 g0[3], g1[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    const T bmin = T(b[d] - s.min[d]);
    const T bmax = T(b[3 + d] - s.min[d]);
    if (bmin < -tol || bmax > s.size[d] + tol)
      return 0;
    const R r = Raster<R, T>::rast(s, d);
    const R mn = R(bmin) * r, mx = R(bmax) * r;
    g0[d] = to_grid(mn < zero ? zero : (maxR < mn ? maxR : mn)); // std::clamp
    g1[d] = to_grid(mx < zero ? zero : (maxR < mx ? maxR : mx));
    if (g0[d] >= res)
      return kBadRegularBox;
    if ((g0[d] != g1[d] && floor(mx) == mx) || g1[d] >= res)
      --g1[d];
  }
  const u64 l0 = encode3(g0[0], g0[1], g0[2]), l1 = encode3(g1[0], g1[1], g1[2]);
  if (l0 == l1)
    return (l0 << 5) | u64(D);
  const u64 diff = l0 ^ l1;
  const u32 levelID = (64u - u32(__clzll((long long)diff)) + 2u) / 3u;
  const u32 shift = 3u * levelID;
  return (((l0 >> shift) << shift) << 5) | u64(D - levelID);
}

template<typename T>
__device__ __forceinline__ u64 regular_box_key(const T* b, const Space<T>& s, u32 D)
{
  return s.rasterDouble ? regular_box_key_ref<T, double>(b, s, D) : regular_box_key_ref<T, float>(b, s, D);
}

// si_grid.h:221-285 GetLooseBoxGridData<2.0> + si_mortongrid.h:78-88 -> loc << 5 | depth
template<typename T, typename R>
__device__ __forceinline__ u64 loose_box_key_ref(const T* b, const Space<T>& s, u32 D)
{
  const T tol = base_tol<T>();
#pragma unroll
  for (int d = 0; d < 3; ++d) // DoesRangeContainBoxAD(space, box, tol), internal_geometry_module.h:214-225
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
    g[d] = center_cell_ref<T, R>(center, s, d);
    maxRel = smax(maxRel, rel_size_ref<T, R>(bsize, s, d));
  }
  u32 maxRelGrid = to_grid(ceil(maxRel));
  u32 level = 0;
  if (maxRelGrid != 0)
    level = 32u - __clz(maxRelGrid - 1u); // std::bit_width
  const u32 shift = level * 3u;
  u64 loc = encode3(g[0], g[1], g[2]);
  loc = shift < 64 ? ((loc >> shift) << shift) : 0;
  return (loc << 5) | u64(u32(D - level));
}

template<typename U>
__device__ __forceinline__ u32 level_from_table(const U* __restrict__ thr, U o)
{
  u32 lo = 0, hi = kLevelThresholds; // thr[0] = 0 <= o
  while (hi - lo > 1)
  {
    u32 m = (lo + hi) >> 1;
    if (o < thr[m])
      hi = m;
    else
      lo = m;
  }
  return lo;
}

__device__ __forceinline__ float to_f(double v) { return __double2float_rn(v); }
__device__ __forceinline__ float to_f(float v) { return v; }

// Location key of one entity from the threshold tables (layout in otg_raster.cuh): integer
// compares only, around an FP32 estimate of the cell.
// Margin of the FP32 cell estimate est = (approx_f(x) - float(min)) * float(rast) of a point
// coordinate x inside the space, against the reference's cell value v = (x - min) * rast (FP64, or
// FP32 for FP32 trees below depth 16). approx_f truncates to 23 mantissa bits (relative error
// below 2^-23), float(min) and float(rast) round to nearest (2^-24 each), and the subtraction and
// the product round to nearest (2^-24 each). With M = max(|min|, |max|) and est, v below `cells`:
//   |est - v| <= rast * M * (2^-23 + 2^-24) + cells * 3 * 2^-24 (+ the reference's own 2^-52 terms)
//             <  rast * M * 2^-22 + cells * 2^-22 + 2^-20.
// A coordinate whose estimate lies more than that margin from every integer, inside (0, cells),
// has the reference's cell trunc(est) and lies inside the space, so it needs no threshold lookup.
// Margins of 1/4 or more switch the shortcut off (2.0 never passes). One thread per dimension.
template<typename T>
__device__ __forceinline__ float cell_estimate_margin(const Space<T>& s, int d, double rast, u32 cells)
{
  const double M = fmax(fabs(double(s.min[d])), fabs(double(s.max[d])));
  const double m = rast * M * 0x1p-22 + double(cells) * 0x1p-22 + 0x1p-20;
  return m < 0.25 ? __double2float_ru(m) : 2.0f;
}

// NARROW (points with 32-bit keys, depth up to 10): the Morton code in 32-bit arithmetic.
// margF (points, optional): the cell-estimate margins of cell_estimate_margin; coordinates whose
// estimates clear them take their cell from the estimate, the others from the threshold tables.
template<typename T, bool IS_BOX, bool NARROW = false>
__device__ __forceinline__ u64 entity_key(const T* e, const typename Ord<T>::U* __restrict__ tab, size_t perDim, u32 cells, const float* minF,
                                          const float* rastF, u32 D, const float* margF = nullptr)
{
  using O = Ord<T>;
  using U = typename O::U;
  if constexpr (!IS_BOX)
  {
    float est[3];
    bool clear = margF != nullptr;
    u32 g[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      est[d] = (approx_f(e[d]) - minF[d]) * rastF[d];
      if (margF)
      {
        const float m = margF[d];
        const bool inside = est[d] > m && est[d] < float(cells) - m;
        g[d] = inside ? u32(est[d]) : 0u;
        const float f = est[d] - float(g[d]);
        clear = clear && inside && f > m && f < 1.0f - m;
      }
    }
    if (clear)
    {
      if constexpr (NARROW)
        return u64(encode3_10(g[0], g[1], g[2]) + 1u);
      else
        return encode3(g[0], g[1], g[2]) + 1;
    }
    bool valid = true;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      const U* td = tab + d * perDim;
      const U o = ord_bits(e[d]);
      valid = valid && o >= td[0] && o <= td[1];
      g[d] = cell_from_table(td + 2 + kLevelThresholds, cells, o, est[d] > 2.0e9f ? 2000000000 : int(est[d]));
    }
    if constexpr (NARROW)
      return valid ? u64(encode3_10(g[0], g[1], g[2]) + 1u) : 0;
    else
      return valid ? encode3(g[0], g[1], g[2]) + 1 : 0;
  }
  else
  {
    bool valid = true;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      const U* td = tab + d * perDim;
      const U lo = ord_bits(e[d]), hi = ord_bits(e[3 + d]);
      valid = valid && lo >= td[0] && lo <= td[1] && hi >= td[0] && hi <= td[1];
    }
    if (!valid)
      return 0;
    u32 g[3], level = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      const U* td = tab + d * perDim;
      const T center = (e[d] + e[3 + d]) * T(0.5); // internal_geometry_module.h:132-138
      const T bsize = T(e[3 + d] - e[d]);           // internal_geometry_module.h:140-146
      const float est = (approx_f(center) - minF[d]) * rastF[d];
      g[d] = cell_from_table(td + 2 + kLevelThresholds, cells, ord_bits(center), est > 2.0e9f ? 2000000000 : int(est));
      level = max(level, level_from_table(td + 2, ord_bits(bsize)));
    }
    const u32 shift = level * 3u;
    u64 loc = encode3(g[0], g[1], g[2]);
    loc = shift < 64 ? ((loc >> shift) << shift) : 0;
    return (loc << 5) | u64(u32(D - level));
  }
}

// STAGED (16-byte aligned entities): whole tiles of 256 chunks (12 KB) arrive in shared memory by
// bulk copies (cp.async.bulk, completion on an mbarrier), two buffers deep, while the previous tile
// is coded; each thread reads its 48-byte chunk from shared memory. The chunks after the last whole
// tile take the direct loads. stageOff: byte offset of the two buffers in dynamic shared memory.
constexpr u32 kCodegenTileChunks = 256;
constexpr u32 kCodegenTileBytes = kCodegenTileChunks * 48;
template<typename T, typename R, typename K, bool IS_BOX, bool STAGED = false>
__global__ void __launch_bounds__(256) codegen_kernel(const T* __restrict__ ent, u64 n, bool vec, const Space<T>* __restrict__ spg,
                                                      const typename Ord<T>::U* __restrict__ tabG, u32 cells, int tabInSmem,
                                                      K* __restrict__ keys, u32* __restrict__ hist, u32 passes, bool regular, u32* __restrict__ err,
                                                      u32 stageOff = 0)
{
  using O = Ord<T>;
  using U = typename O::U;
  constexpr int W = IS_BOX ? 6 : 3;
  constexpr int E = Chunk<T, W>::E;
  extern __shared__ __align__(16) unsigned char s_dyn[];
  __shared__ u32 sh[8][kRadix];
  __shared__ float minF[3], rastF[3], margF[3];
  __shared__ u32 sD;
  const size_t perDim = RasterLayout<T>::per_dim(cells);
  U* stab = reinterpret_cast<U*>(s_dyn);
  for (int i = threadIdx.x; i < 8 * kRadix; i += blockDim.x)
    (&sh[0][0])[i] = 0;
  if (tabInSmem)
    for (size_t i = threadIdx.x; i < 3 * perDim; i += blockDim.x)
      stab[i] = tabG[i];
  if (threadIdx.x < 3)
  {
    const Space<T>& s = *spg;
    minF[threadIdx.x] = to_f(s.min[threadIdx.x]);
    rastF[threadIdx.x] = float(Raster<R, T>::rast(s, threadIdx.x));
    margF[threadIdx.x] = cell_estimate_margin(s, threadIdx.x, double(Raster<R, T>::rast(s, threadIdx.x)), cells);
    if (threadIdx.x == 0)
      sD = s.D;
  }
  __syncthreads();
  const U* tab = tabInSmem ? stab : tabG;
  const u32 D = sD;
  const u64 chunks = (n + E - 1) / E;
  auto code = [&](const T* v, u64 c, int cnt) {
#pragma unroll
    for (int k = 0; k < E; ++k)
    {
      if (k >= cnt)
        break;
      K kk;
      if constexpr (IS_BOX)
      {
        u64 k64 = regular ? regular_box_key<T>(v + k * W, *spg, D) : entity_key<T, IS_BOX>(v + k * W, tab, perDim, cells, minF, rastF, D);
        if (k64 == kBadRegularBox)
        {
          atomicOr(err, kErrArgument);
          k64 = 0;
        }
        kk = K(k64);
      }
      else
        kk = K(entity_key<T, IS_BOX, sizeof(K) == 4>(v + k * W, tab, perDim, cells, minF, rastF, D, margF));
      keys[c * E + k] = kk;
      for (u32 p = 0; p < passes; ++p)
        atomicAdd(&sh[p][(kk >> (kRadixBits * p)) & (kRadix - 1)], 1u);
    }
  };
  u64 firstDirect = 0;
  if constexpr (STAGED)
  {
    __shared__ __align__(8) u64 s_bar[2];
    unsigned char* stage = s_dyn + stageOff;
    const u64 fullTiles = chunks == 0 ? 0 : (n / E) / kCodegenTileChunks; // tiles of whole chunks only
    const unsigned char* src = reinterpret_cast<const unsigned char*>(ent);
    if (threadIdx.x == 0)
    {
      mbar_init(&s_bar[0], 1);
      mbar_init(&s_bar[1], 1);
      fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](u64 tile, int b) {
      mbar_arrive_expect_tx(&s_bar[b], kCodegenTileBytes);
      bulk_load(stage + b * kCodegenTileBytes, src + tile * kCodegenTileBytes, kCodegenTileBytes, &s_bar[b]);
    };
    u64 t = blockIdx.x;
    u32 it = 0;
    if (threadIdx.x == 0 && t < fullTiles)
      issue(t, 0);
    bool failed = false;
    for (; t < fullTiles; t += gridDim.x, ++it)
    {
      const int b = int(it & 1u);
      if (threadIdx.x == 0 && t + gridDim.x < fullTiles)
      {
        fence_proxy_async(); // buffer b ^ 1 was read before the barrier that ended the last tile
        issue(t + gridDim.x, b ^ 1);
      }
      const bool ok = mbar_wait_bounded(&s_bar[b], (it >> 1) & 1u);
      if (__syncthreads_or(!ok))
      {
        failed = true;
        break;
      }
      T v[E * W];
      const T* mine = reinterpret_cast<const T*>(stage + b * kCodegenTileBytes) + threadIdx.x * (E * W);
      if constexpr (sizeof(T) == 8)
      {
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
          const double2 x = reinterpret_cast<const double2*>(mine)[j];
          v[2 * j] = x.x;
          v[2 * j + 1] = x.y;
        }
      }
      else
      {
#pragma unroll
        for (int j = 0; j < 3; ++j)
        {
          const float4 x = reinterpret_cast<const float4*>(mine)[j];
          v[4 * j] = x.x;
          v[4 * j + 1] = x.y;
          v[4 * j + 2] = x.z;
          v[4 * j + 3] = x.w;
        }
      }
      code(v, t * kCodegenTileChunks + threadIdx.x, E);
      __syncthreads(); // buffer b is read: the copy two tiles on may overwrite it
    }
    if (failed)
    {
      // the copies in flight land before this block's shared memory goes away; the error bit fails
      // the build
      if (threadIdx.x == 0)
        atomicOr(err, kErrTimeout);
      mbar_wait_bounded(&s_bar[it & 1u], (it >> 1) & 1u);
      mbar_wait_bounded(&s_bar[(it + 1) & 1u], ((it + 1) >> 1) & 1u);
      return;
    }
    firstDirect = fullTiles * kCodegenTileChunks;
  }
  for (u64 c = firstDirect + blockIdx.x * u64(blockDim.x) + threadIdx.x; c < chunks; c += u64(gridDim.x) * blockDim.x)
  {
    T v[E * W];
    const int cnt = load_chunk<T, W>(ent, n, c * E, vec, v);
    code(v, c, cnt);
  }
  __syncthreads();
  for (u32 p = 0; p < passes; ++p)
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
      if (sh[p][d])
        atomicAdd(&hist[p * kRadix + d], sh[p][d]);
}

// per-entity location keys in input order, reference layout (loc << 5 | depth), computed with the
// reference formulas from the tree-ordered copy
template<typename T, typename R, bool IS_BOX>
__global__ void location_export_kernel(const T* __restrict__ geom, const u32* __restrict__ ids, u64 n, const Space<T>* __restrict__ spg,
                                       u64* __restrict__ out, bool regular)
{
  const Space<T> s = *spg;
  const u32 D = s.D;
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    const u32 id = ids[i];
    if (id >= n)
      continue;
    if constexpr (IS_BOX)
      out[id] = regular ? regular_box_key_ref<T, R>(geom + i * 6, s, D) : loose_box_key_ref<T, R>(geom + i * 6, s, D);
    else
    {
      u64 k = point_key_ref<T, R>(geom + i * 3, s, (1u << D) - 1u);
      out[id] = k == 0 ? 0 : (((k - 1) << 5) | D);
    }
  }
}

// ---------------------------------------------------------------- 5. gather into tree order
// Random reads of whole entities: every thread issues the loads of kGatherPerThread entities
// before storing any of them, so many sectors are in flight per thread.
constexpr int kGatherPerThread = 4;
constexpr int kGatherWide = 8; // the single-tree gather that runs beside the emission

template<typename T, int W, int G>
__global__ void __launch_bounds__(256) gather_kernel(const T* __restrict__ ent, const u32* __restrict__ ids, u64 n, T* __restrict__ out)
{
  constexpr int kGatherPerThread = G;
  const u64 stride = u64(gridDim.x) * blockDim.x;
  for (u64 i0 = blockIdx.x * u64(blockDim.x) + threadIdx.x; i0 < n; i0 += stride * kGatherPerThread)
  {
    T v[kGatherPerThread][W];
    u32 id[kGatherPerThread];
#pragma unroll
    for (int k = 0; k < kGatherPerThread; ++k)
    {
      const u64 i = i0 + k * stride;
      id[k] = i < n ? ids[i] : 0xffffffffu;
    }
#pragma unroll
    for (int k = 0; k < kGatherPerThread; ++k)
      if (id[k] < n)
#pragma unroll
        for (int c = 0; c < W; ++c)
          v[k][c] = ent[u64(id[k]) * W + c];
#pragma unroll
    for (int k = 0; k < kGatherPerThread; ++k)
    {
      const u64 i = i0 + k * stride;
      if (i < n && id[k] < n)
#pragma unroll
        for (int c = 0; c < W; ++c)
          out[i * W + c] = v[k][c];
    }
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


template<typename T>
__global__ void root_init_kernel(uint4* link, u64* nodeKey, unsigned char* nodeDepth, u32* levelCount, u32 n, u32* nodeParent)
{
  if (threadIdx.x == 0 && blockIdx.x == 0)
  {
    link[0] = make_uint4(0, 0, 0, n);
    nodeKey[0] = 1;
    nodeDepth[0] = 0;
    levelCount[0] = 1;
    if (nodeParent)
      nodeParent[0] = 0;
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

// MinPoint of a node from the table (identical arithmetic, computed once per cell), dimension dim
template<typename T>
__device__ __forceinline__ void write_min_point(T* nodeBox, u32 node, u64 key, u32 d, int dim, const T* minTab, u64 tabPerDim, const Space<T>* spg)
{
  const u64 loc = key ^ (u64(1) << (3 * d));
  const u32 cell = compact1by2(loc >> dim);
  T* nb = nodeBox + u64(node) * 6;
  nb[dim] = minTab[u64(dim) * tabPerDim + ((u64(1) << d) - 1) + cell];
  nb[3 + dim] = spg->nodeSize[d][dim];
}

// MinPoint and size of a node in all three dimensions, as three 16-byte (FP64) or 8-byte (FP32) stores
template<typename T>
__device__ __forceinline__ void write_node_min(T* nodeBox, u32 node, u64 key, u32 d, const T* minTab, u64 tabPerDim, const T (*size)[3])
{
  const u64 loc = key ^ (u64(1) << (3 * d));
  T v[6];
#pragma unroll
  for (int dim = 0; dim < 3; ++dim)
  {
    v[dim] = minTab[u64(dim) * tabPerDim + ((u64(1) << d) - 1) + compact1by2(loc >> dim)];
    v[3 + dim] = size[d][dim];
  }
  using V2 = typename std::conditional<sizeof(T) == 8, double2, float2>::type;
  V2* p = reinterpret_cast<V2*>(nodeBox + u64(node) * 6);
  p[0] = V2{v[0], v[1]};
  p[1] = V2{v[2], v[3]};
  p[2] = V2{v[4], v[5]};
}

// emit_classify_kernel, one thread per node, decides the roots: a node that does not split (at most
// maxElem entities in its subtree, or d == maxDepth) keeps all of them and is finished at once
// (ProcessNode, :656-683); a node that splits goes to a queue. Then one emit_split_kernel launch per
// depth, eight lanes per queued node, which also decides each child it creates (leaf now, or the
// next depth's queue, of two alternating queue buffers): lane 0 finds the end of the node's stuck entities (ProcessNode's
// partition_point, :658-671) and lanes 1..7 the start of child key ranges 1..7
// (CreateProcessingData's partition_point, :695-711) at the same time, so the dependent-load
// chain of a node is one binary search deep. Below the root every key of a node's range shares
// its prefix, so child 7 ends where the range ends; at the root lane 0 also searches that end
// (locations outside the 3*D-bit grid sort after every child range and belong to no child).
// Per-tree parameters of a forest build (several independent trees emitted together: node t is
// the root of tree t). All null for a single tree.
struct ForestNodes
{
  u32* nodeTree;     // tree of each node
  const u32* treeD;  // max depth of each tree
  const u64* minOff; // offset of each tree's MinPoint table (point trees)
};

// the depth, space and MinPoint table of the tree that holds `node`
template<typename T>
__device__ __forceinline__ void node_tree_params(const ForestNodes& fn, u32 node, u32& D, const Space<T>*& sp, const T*& minTab)
{
  if (fn.nodeTree)
  {
    const u32 tr = fn.nodeTree[node];
    D = fn.treeD[tr];
    sp += tr;
    if (fn.minOff)
      minTab += fn.minOff[tr];
  }
}

template<typename T, bool IS_BOX>
__global__ void __launch_bounds__(256) emit_classify_kernel(u32 d, u32 D, u64 maxElem, uint4* __restrict__ link, const u64* __restrict__ nodeKey,
                                                            T* __restrict__ nodeBox, const u32* __restrict__ levelCount, u32* __restrict__ splitCount,
                                                            u32* __restrict__ splitQueue, u32 queueCap, const T* __restrict__ minTab,
                                                            const Space<T>* __restrict__ spg, u32* __restrict__ ownerNode, u32* __restrict__ err,
                                                            ForestNodes fn)
{
  u32 begin, cnt;
  level_range(levelCount, d, begin, cnt);
  const int lane = threadIdx.x & 31;
  for (u32 i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < cnt; i0 += gridDim.x * blockDim.x)
  {
    const u32 i = i0 + lane;
    bool split = false;
    u32 node = 0;
    if (i < cnt)
    {
      node = begin + i;
      u32 Dn = D;
      const Space<T>* spn = spg;
      const T* mt = minTab;
      node_tree_params(fn, node, Dn, spn, mt);
      const uint4 L = link[node];
      split = u64(L.w - L.y) > maxElem && d < Dn;
      if (!split)
      {
        link[node] = make_uint4(0, L.y, L.w, L.w);
        if (ownerNode)
          for (u32 q = L.y; q < L.w; ++q)
            ownerNode[q] = node;
        if constexpr (!IS_BOX)
          write_node_min(nodeBox, node, nodeKey[node], d, mt, (u64(2) << Dn) - 1, spn->nodeSize);
      }
    }
    const u32 m = __ballot_sync(0xffffffffu, split);
    u32 qb = 0;
    if (lane == 0 && m)
      qb = atomicAdd(&splitCount[d], __popc(m));
    qb = __shfl_sync(0xffffffffu, qb, 0);
    if (split)
    {
      const u32 slot = qb + __popc(m & lanemask_lt());
      if (slot < queueCap) // a node that splits holds more than maxElem entities: at most n / (maxElem + 1) per depth
        splitQueue[slot] = node;
      else
        atomicOr(err, kErrCapacity);
    }
  }
}

constexpr u32 kEmitCountMax = 256;

template<typename T, typename K, bool IS_BOX>
__global__ void __launch_bounds__(256) emit_split_kernel(u32 d, u32 D, const K* __restrict__ keys, uint4* __restrict__ link, u64* __restrict__ nodeKey,
                                                         T* __restrict__ nodeBox, unsigned char* __restrict__ nodeDepth, u32* __restrict__ levelCount,
                                                         u32* __restrict__ splitCount, const u32* __restrict__ splitQueue, u32 queueCap,
                                                         const T* __restrict__ minTab, const Space<T>* __restrict__ spg, u64 maxNodes, u32* __restrict__ err,
                                                         u32* __restrict__ ownerNode, u32* __restrict__ nodeParent, ForestNodes fn, u64 maxElem,
                                                         u32* __restrict__ queueOut)
{
  u32 begin, cnt;
  level_range(levelCount, d, begin, cnt);
  const u32 childBase = begin + cnt;
  const u32 qcount = min(splitCount[d], queueCap);
  const int lane = threadIdx.x & 31;
  const int grp = lane >> 3, gl = lane & 7;
  const u32 groupMask = 0xffu << (grp * 8);
  const u32 warpGlobal = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const u32 warpsTotal = (gridDim.x * blockDim.x) >> 5;
  const u32 D0 = D;
  for (u32 qbase = warpGlobal * 4; qbase < qcount; qbase += warpsTotal * 4)
  {
    const u32 qi = qbase + grp;
    const bool active = qi < qcount;
    const u32 node = active ? splitQueue[qi] : 0;
    u32 b = 0, e = 0, bnd = 0, end8 = 0;
    u64 key = 1;
    // the tree of this group's node: its depth, space and MinPoint table
    u32 D = D0;
    const Space<T>* spn = spg;
    const T* mt = minTab;
    u32 tree = 0;
    if (active)
    {
      node_tree_params(fn, node, D, spn, mt);
      if (fn.nodeTree)
        tree = fn.nodeTree[node];
    }
    const u64 tabPerDim = (u64(2) << D) - 1;
    if (active)
    {
      const uint4 L = link[node];
      key = nodeKey[node];
      b = L.y;
      e = L.w;
      end8 = e;
    }
    // small ranges: the group reads the range once and counts keys per child (coalesced, two
    // round trips); large ranges (upper depths): one binary search per lane
    const bool small = active && d > 0 && (e - b) <= kEmitCountMax; // uniform within a group
    if (__any_sync(0xffffffffu, small))
    {
      // all lanes run the counting loop and the shuffles; groups that are not small count nothing
      const u32 shiftChild = 3 * (D - d - 1);
      u32 below[8]; // keys of this lane with child index < c (c = 1..7), and stuck keys in [0]
#pragma unroll
      for (int c = 0; c < 8; ++c)
        below[c] = 0;
      const u64 lmin = (key ^ (u64(1) << (3 * d))) << (3 * (D - d));
      // four keys per lane in flight per round: the loads of a round are independent
      for (u32 q0 = b + gl; small && q0 < e; q0 += 32)
      {
        K kq[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          kq[u] = q0 + 8 * u < e ? keys[q0 + 8 * u] : K(0);
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
          if (q0 + 8 * u >= e)
            break;
          const u64 k = u64(kq[u]);
          if constexpr (IS_BOX)
          {
            const bool stuck = k <= ((lmin << 5) | u64(d));
            below[0] += stuck ? 1u : 0u;
            const u32 c = stuck ? 0u : u32(((k >> 5) >> shiftChild) & 7u);
#pragma unroll
            for (int cc = 1; cc < 8; ++cc)
              below[cc] += (stuck || c < u32(cc)) ? 1u : 0u;
          }
          else
          {
            const u32 c = u32(((k - 1) >> shiftChild) & 7u);
#pragma unroll
            for (int cc = 1; cc < 8; ++cc)
              below[cc] += c < u32(cc) ? 1u : 0u;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 8; ++c)
      {
        u32 v = below[c];
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        below[c] = v;
      }
      u32 mine = below[0];
#pragma unroll
      for (int c = 1; c < 8; ++c)
        mine = gl == c ? below[c] : mine;
      if (small)
        bnd = b + mine;
    }
    if (active && !small)
    {
      const u64 lmin = (key ^ (u64(1) << (3 * d))) << (3 * (D - d));
      const u64 S = u64(1) << (3 * (D - d - 1));
      if (gl == 0)
      {
        if constexpr (IS_BOX)
          bnd = upper_bound_key(keys, b, e, (lmin << 5) | u64(d));
        else
          bnd = (d == 0) ? upper_bound_key(keys, b, e, 0) : b;
        if (d == 0)
        {
          const u64 L8 = lmin + 8 * S;
          end8 = lower_bound_key(keys, bnd, e, IS_BOX ? (L8 << 5) : (L8 + 1));
        }
      }
      else
      {
        const u64 L0 = lmin + u64(gl) * S;
        bnd = lower_bound_key(keys, b, e, IS_BOX ? (L0 << 5) : (L0 + 1));
      }
    }
    const u32 end8g = __shfl_sync(0xffffffffu, end8, grp * 8);
    const u32 myStart = bnd;                                            // lane c: start of child c (lane 0: stuck end)
    const u32 nextLane = __shfl_sync(0xffffffffu, bnd, (lane + 1) & 31); // lane c: start of child c + 1
    const u32 nextStart = gl < 7 ? nextLane : end8g;
    const bool nonEmpty = active && nextStart > myStart;
    const u32 ballot = __ballot_sync(0xffffffffu, nonEmpty) & groupMask;
    const u32 nchild = __popc(ballot);
    const u32 ownEnd = __shfl_sync(0xffffffffu, bnd, grp * 8);
    // warp-aggregated allocation of the children slots (children of one node are contiguous)
    const u32 mine = (gl == 0) ? nchild : 0u;
    u32 incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      u32 y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o)
        incl += y;
    }
    const u32 warpTotal = __shfl_sync(0xffffffffu, incl, 31);
    u32 warpBase = 0;
    if (lane == 31 && warpTotal)
      warpBase = atomicAdd(&levelCount[d + 1], warpTotal);
    warpBase = __shfl_sync(0xffffffffu, warpBase, 31);
    const u32 firstChild = childBase + warpBase + __shfl_sync(0xffffffffu, incl - mine, grp * 8);
    const bool overflow = u64(firstChild) + nchild > maxNodes;
    u32 ci = 0;
    bool enq = false;
    if (active)
    {
      if (nonEmpty && !overflow)
      {
        ci = firstChild + __popc(ballot & lanemask_lt());
        const u64 ckey = (key << 3) | u64(gl);
        nodeKey[ci] = ckey;
        nodeDepth[ci] = (unsigned char)(d + 1);
        if (nodeParent)
          nodeParent[ci] = node;
        if (fn.nodeTree)
          fn.nodeTree[ci] = tree;
        // the child's own split decision (ProcessNode, :656-683), made here instead of by a
        // classify launch at the next depth: a child that splits goes to the next depth's queue
        // and gets its children there; one that does not keeps all its entities now
        enq = u64(nextStart - myStart) > maxElem && d + 1 < D;
        if (enq)
          link[ci] = make_uint4(0, myStart, myStart, nextStart);
        else
        {
          link[ci] = make_uint4(0, myStart, nextStart, nextStart);
          if (ownerNode)
            for (u32 q = myStart; q < nextStart; ++q)
              ownerNode[q] = ci;
          if constexpr (!IS_BOX)
            write_node_min(nodeBox, ci, ckey, d + 1, mt, tabPerDim, spn->nodeSize);
        }
      }
      if (gl == 0)
      {
        if (overflow)
          atomicOr(err, kErrCapacity);
        const u32 nc = overflow ? 0u : nchild;
        link[node] = make_uint4((nc ? (firstChild & kFirstChildMask) : 0u) | (nc << kChildShift), b, ownEnd, e);
      }
      if (ownerNode)
        for (u32 q = b + gl; q < ownEnd; q += 8)
          ownerNode[q] = node;
      if constexpr (!IS_BOX)
        if (gl < 3)
          write_min_point(nodeBox, node, key, d, gl, mt, tabPerDim, spn);
    }
    // warp-aggregated append of the children that split
    const u32 qm = __ballot_sync(0xffffffffu, enq);
    if (qm)
    {
      u32 qb0 = 0;
      if (lane == 0)
        qb0 = atomicAdd(&splitCount[d + 1], u32(__popc(qm)));
      qb0 = __shfl_sync(0xffffffffu, qb0, 0);
      if (enq)
      {
        const u32 slot = qb0 + __popc(qm & lanemask_lt());
        if (slot < queueCap)
          queueOut[slot] = ci;
        else
          atomicOr(err, kErrCapacity);
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
// One block per root (node r is the root of tree r in a forest; a single tree has root 0).
template<typename T>
__global__ void __launch_bounds__(256) root_box_kernel(const uint4* __restrict__ link, const T* __restrict__ sortedGeom, T* __restrict__ nodeBox,
                                                       Space<T>* spAll)
{
  __shared__ T smn[3][256], smx[3][256];
  const u32 root = blockIdx.x;
  Space<T>* sp = spAll + root;
  nodeBox += u64(root) * 6;
  const uint4 L = link[root];
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
// The single-tree sort: decoupled look-back passes (otg_sort.cuh), or with OTG_SORT=chunked the
// chunked persistent passes (otg_sort_chunked.cuh); forests and recorded builds use the former.
static bool chunked_sort_enabled()
{
  static const bool on = [] {
    const char* v = std::getenv("OTG_SORT");
    return v && std::strcmp(v, "chunked") == 0;
  }();
  return on;
}
// widest digit of the chunked passes (OTG_SORT_BITS, 8-11)
static int chunked_sort_bits()
{
  static const int b = [] {
    const char* v = std::getenv("OTG_SORT_BITS");
    return v ? std::atoi(v) : kChunkMaxBits;
  }();
  return b;
}

static int grid_blocks(u64 n, int perBlock = 256, int maxBlocks = 152 * 16)
{
  u64 b = (n + perBlock - 1) / perBlock;
  return int(std::max<u64>(1, std::min<u64>(b, u64(maxBlocks))));
}

// Grid of one emission launch at depth d: `roots` trees hold at most roots * 8^d nodes there, and
// splitting ones are also bounded by the queue; `perBlock` nodes per 256-thread block.
static int emit_blocks(u32 d, u64 roots, int maxBlocks, u64 queueCap, u64 perBlock)
{
  const u64 cap = std::min<u64>(d < 20 ? roots << (3 * d) : ~u64(0), queueCap);
  return int(std::max<u64>(1, std::min<u64>(u64(maxBlocks), (cap + perBlock - 1) / perBlock)));
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

// The emission stream of a tree (highest priority: the emission's launches are short and dependent,
// so they go first when both streams have work) and its fork / join events, created on first use,
// which is always an ordinary build, never a recorded one.
static int emission_stream(TreeState& t, cudaStream_t& es)
{
  if (!t.side)
  {
    int lowest = 0, highest = 0;
    cudaDeviceGetStreamPriorityRange(&lowest, &highest);
    cudaError_t e;
    if ((e = cudaStreamCreateWithPriority(&t.side, cudaStreamNonBlocking, highest)) || (e = cudaEventCreateWithFlags(&t.fork, cudaEventDisableTiming)) ||
        (e = cudaEventCreateWithFlags(&t.join, cudaEventDisableTiming)))
      return cuda_status(e, "creating the emission stream");
  }
  es = t.side;
  return OTG_OK;
}

template<typename T, typename K, bool IS_BOX>
// pull (optional): the entities in pinned host memory, mapped for the device; the bounding-box pass
// reads them there and writes the device copy `ent` on the way
static int build_impl(TreeState& t, const T* ent, const void* box, u64 n, cudaStream_t st, const T* pull = nullptr)
{
  constexpr int W = IS_BOX ? 6 : 3;
  using U = typename Ord<T>::U;
  const bool regular = t.kind == OTG_KIND_BOXES_REGULAR; // GetBoxGridID instead of the loose grid data
  const u32 D = t.D;
  const u32 bits = IS_BOX ? 3 * D + 5 : 3 * D + 1;
  const bool chunked = chunked_sort_enabled();
  // histogram passes computed by codegen: the onesweep passes need them, the chunked ones count
  // their own digits
  // sorted key bits: a loose box centred on the max face of its space has the out-of-grid cell 2^D
  // in up to three dimensions, so its key can hold three bits above 3D + 5
  const u32 sortBits = IS_BOX ? std::min(3 * D + 8, u32(8 * sizeof(K))) : bits;
  const u32 passes = chunked ? 0u : (sortBits + kRadixBits - 1) / kRadixBits;
  const u32 cells = IS_BOX ? (1u << D) + 2 : (1u << D);
  const size_t tabBytes = RasterLayout<T>::bytes(cells);
  const u64 minTabEntries = IS_BOX ? 1 : 3 * ((u64(2) << D) - 1);
  cudaError_t e;

  // buffers
  const u64 maxNodes = n + u64(D) * (n / (t.maxElem + 1) + 1) + 2;
  t.maxNodes = maxNodes;
  if ((e = t.keysA.ensure(sizeof(K) * n)) || (e = t.keysB.ensure(sizeof(K) * n)) || (e = t.sortedIds.ensure(sizeof(u32) * n)) ||
      (e = t.valsB.ensure(sizeof(u32) * n)) || (e = t.sortedGeom.ensure(sizeof(T) * W * n)) || (e = t.nodeLink.ensure(sizeof(uint4) * maxNodes)) ||
      (e = t.nodeKey.ensure(sizeof(u64) * maxNodes)) || (e = t.nodeBox.ensure(sizeof(T) * 6 * maxNodes)) ||
      (e = t.nodeDepth.ensure(maxNodes)) || (e = t.levelCount.ensure(sizeof(u32) * 64)) ||
      (e = t.splitQueue.ensure(2 * sizeof(u32) * (n / (t.maxElem + 1) + 2))) || (e = t.space.ensure(sizeof(Space<T>))) ||
      (e = t.sortScratch.ensure(chunked ? ChunkScratch::bytes() : SortScratch::bytes(n, passes))) || (e = t.bboxBits.ensure(sizeof(U) * 6)) ||
      (e = t.rasterTab.ensure(tabBytes)) || (e = t.minTab.ensure(sizeof(T) * minTabEntries)) ||
      (IS_BOX && ((e = t.nodeMax.ensure(sizeof(T) * 3 * maxNodes)) || (e = t.ownerNode.ensure(sizeof(u32) * n)) ||
                  (e = t.nodeParent.ensure(sizeof(u32) * maxNodes)))))
    return cuda_status(e, "allocating tree buffers");

  Profiler& prof = profiler();
  prof.reset();
  prof.mark("setup", st);
  SortScratch ss;
  ChunkScratch cs;
  if (chunked)
  {
    cs.carve(t.sortScratch.p);
    cudaMemsetAsync(static_cast<unsigned char*>(t.sortScratch.p) + ChunkScratch::zero_offset(), 0, ChunkScratch::zero_bytes(), st);
  }
  else
  {
    ss.carve(t.sortScratch.p, n, passes);
    cudaMemsetAsync(t.sortScratch.p, 0, SortScratch::bytes(n, passes), st);
  }
  cudaMemsetAsync(t.levelCount.p, 0, sizeof(u32) * 64, st);

  const bool vec = (reinterpret_cast<uintptr_t>(ent) & 15) == 0;
  Space<T>* sp = t.space.as<Space<T>>();
  if (!box)
  {
    prof.mark("bbox", st);
    bbox_init_kernel<U><<<1, 32, 0, st>>>(t.bboxBits.as<U>());
    // up to 16 blocks per SM (16M points: 0.0925 ms at 8 per SM, 0.088 ms at 16)
    if (pull)
      pull_bbox_kernel<T, W><<<grid_blocks(n * W * sizeof(T) / 16 + 1, 256, 152 * 16), 256, 0, st>>>(pull, n, const_cast<T*>(ent),
                                                                                                      t.bboxBits.as<U>());
    else
      bbox_kernel<T, W><<<grid_blocks((n + Chunk<T, W>::E - 1) / Chunk<T, W>::E, 256, 152 * 16), 256, 0, st>>>(ent, n, vec, t.bboxBits.as<U>());
  }
  prof.mark("tables", st);
  space_setup_kernel<T><<<1, 1, 0, st>>>(sp, t.bboxBits.as<U>(), (const T*)box, D, IS_BOX ? 0 : 1);
  const bool rasterDouble = (sizeof(T) == 8) || D >= 16;
  U* tab = t.rasterTab.as<U>();
  const u64 tabEntries = 3 * RasterLayout<T>::per_dim(cells);
  if (rasterDouble)
    raster_tables_kernel<T, double><<<grid_blocks(tabEntries, 128, 152 * 32), 128, 0, st>>>(sp, tab, cells, IS_BOX ? 1 : 0);
  else
    raster_tables_kernel<T, float><<<grid_blocks(tabEntries, 128, 152 * 32), 128, 0, st>>>(sp, tab, cells, IS_BOX ? 1 : 0);
  if constexpr (!IS_BOX)
  {
    if (rasterDouble)
      node_min_table_kernel<T, double><<<grid_blocks(minTabEntries), 256, 0, st>>>(sp, t.minTab.as<T>());
    else
      node_min_table_kernel<T, float><<<grid_blocks(minTabEntries), 256, 0, st>>>(sp, t.minTab.as<T>());
  }

  prof.mark("codegen", st);
  const int tabInSmem = tabBytes <= 64 * 1024 ? 1 : 0;
  static const bool cgStage = [] {
    const char* v = std::getenv("OTG_CODEGEN_STAGE");
    return v && v[0] == '1';
  }();
  const bool staged = cgStage && vec;
  const u32 stageOff = u32((tabInSmem ? tabBytes : 0) + 15) & ~15u;
  const size_t cgSmem = staged ? stageOff + 2 * kCodegenTileBytes : (tabInSmem ? tabBytes : 0);
  // up to 16 blocks per SM: more blocks in flight than fit at once balance the grid-stride loop
  // (16M points: 0.184 ms at 4 per SM, 0.168 ms at 16, 0.186 ms at 64)
  int cgBlocks = grid_blocks((n + Chunk<T, W>::E - 1) / Chunk<T, W>::E, 256, 152 * 16);
  auto kfn = rasterDouble ? (staged ? codegen_kernel<T, double, K, IS_BOX, true> : codegen_kernel<T, double, K, IS_BOX>)
                          : (staged ? codegen_kernel<T, float, K, IS_BOX, true> : codegen_kernel<T, float, K, IS_BOX>);
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(cgSmem));
  if (staged)
  {
    // the tiles are shared out over the blocks that fit at once
    int perSm = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kfn, 256, cgSmem);
    cgBlocks = std::max(1, std::min(cgBlocks, std::max(perSm, 1) * std::max(sms, 1)));
  }
  kfn<<<cgBlocks, 256, cgSmem, st>>>(ent, n, vec, sp, tab, cells, tabInSmem, t.keysA.as<K>(), ss.hist, passes, regular, t.err.as<u32>(), stageOff);

  prof.mark("sort", st);
  bool inB = false;
  if (chunked)
  {
    if (int rc = chunk_sort<K>(t.keysA.as<K>(), t.sortedIds.as<u32>(), t.keysB.as<K>(), t.valsB.as<u32>(), n, sortBits, true, cs, t.err.as<u32>(), st,
                               &inB, chunked_sort_bits()))
      return rc;
  }
  else
    inB = onesweep_passes<K>(t.keysA.as<K>(), t.sortedIds.as<u32>(), t.keysB.as<K>(), t.valsB.as<u32>(), n, 0, passes, true, ss, t.err.as<u32>(), st);
  if (inB)
  {
    std::swap(t.sortedIds, t.valsB);
    t.sortedKeys = t.keysB.p;
  }
  else
    t.sortedKeys = t.keysA.p;
  const K* keys = reinterpret_cast<const K*>(t.sortedKeys);

  // Node emission reads only the sorted keys, so it runs on a second stream beside the gather: the
  // gather is bound by DRAM, the emission by the latency of its short dependent launches.
  cudaStream_t es = st;
  if (int rc = emission_stream(t, es))
    return rc;
  // entities that the emission places in no node keep kNoOwner
  if (IS_BOX && (e = cudaMemsetAsync(t.ownerNode.p, 0xff, sizeof(u32) * n, st)))
    return cuda_status(e, "clearing the entity owners");
  if ((e = cudaEventRecord(t.fork, st)) || (e = cudaStreamWaitEvent(es, t.fork, 0)))
    return cuda_status(e, "ordering the emission stream");
  prof.mark("gather+emit", st);
  // Two gather blocks per SM, 8 independent entity loads per thread, leave the rest of each SM to the
  // emission. A full-occupancy gather holds every SM until it ends. Measured beside the emission
  // (16M points): 0.512 ms for this shape, 0.573 ms for one block per SM with 4 loads, 0.587 ms at
  // full occupancy (sweep of 152-2432 blocks and 2-16 loads per thread).
  // Box trees (entities twice as wide): one block per SM with 2 loads per thread, 2.5% faster for the
  // 8M-box rebuild than 4 loads (sweep of 152-608 blocks and 2-4 loads per thread).
  constexpr int G = IS_BOX ? 2 : kGatherWide;
  gather_kernel<T, W, G><<<grid_blocks((n + G - 1) / G, 256, IS_BOX ? 152 : 2 * 152), 256, 0, st>>>(ent, t.sortedIds.as<u32>(), n,
                                                                                                   t.sortedGeom.as<T>());

  u32* parent = IS_BOX ? t.nodeParent.as<u32>() : nullptr;
  const int emitBlocks = grid_blocks(maxNodes, 256, 152 * 16);
  u32* levelCount = t.levelCount.as<u32>();
  u32* splitCount = levelCount + 32;
  u32* splitQueue = t.splitQueue.as<u32>();
  const u32 queueCap = u32(n / (t.maxElem + 1) + 2);
  root_init_kernel<T><<<1, 32, 0, es>>>(t.nodeLink.as<uint4>(), t.nodeKey.as<u64>(), t.nodeDepth.as<unsigned char>(), levelCount, u32(n), parent);
  // the root's decision, then one launch per depth (queues of depths d and d + 1 alternate halves)
  emit_classify_kernel<T, IS_BOX><<<1, 256, 0, es>>>(0, D, t.maxElem, t.nodeLink.as<uint4>(), t.nodeKey.as<u64>(), t.nodeBox.as<T>(), levelCount,
                                                     splitCount, splitQueue, queueCap, t.minTab.as<T>(), sp, IS_BOX ? t.ownerNode.as<u32>() : nullptr,
                                                     t.err.as<u32>(), ForestNodes{});
  for (u32 d = 0; d < D; ++d)
  {
    const int splitBlocks = emit_blocks(d, 1, emitBlocks, queueCap, 32);
    emit_split_kernel<T, K, IS_BOX><<<splitBlocks, 256, 0, es>>>(d, D, keys, t.nodeLink.as<uint4>(), t.nodeKey.as<u64>(), t.nodeBox.as<T>(),
                                                                t.nodeDepth.as<unsigned char>(), levelCount, splitCount, splitQueue + (d & 1) * queueCap,
                                                                queueCap, t.minTab.as<T>(), sp, maxNodes, t.err.as<u32>(),
                                                                IS_BOX ? t.ownerNode.as<u32>() : nullptr, parent, ForestNodes{}, t.maxElem,
                                                                splitQueue + ((d + 1) & 1) * queueCap);
  }
  if ((e = cudaEventRecord(t.join, es)) || (e = cudaStreamWaitEvent(st, t.join, 0)))
    return cuda_status(e, "joining the emission stream");
  prof.mark("geometry", st);
  if constexpr (IS_BOX)
  {
    for (int d = int(D); d >= 0; --d)
      mbr_level_kernel<T><<<emit_blocks(u32(d), 1, emitBlocks, ~u64(0), 256), 256, 0, st>>>(u32(d), t.levelCount.as<u32>(), t.nodeLink.as<uint4>(), t.sortedGeom.as<T>(), t.nodeBox.as<T>(),
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

// The L2 fetch granularity limit of this process's CUDA context (cudaLimitMaxL2FetchGranularity, a
// per-context performance hint that ends with the process). The gather of a build reads one 24-byte
// point at a random position per output, and each such read brings about a whole 128-byte line from
// DRAM (125 B per point measured at 16M points).
// OTG_L2_FETCH_BYTES=b sets the context's L2 fetch granularity limit before the first build (0 or
// unset: unchanged). Measured on the 16M-point build: unchanged 1.359 ms, 32 B 1.394 ms, 64 B
// 1.365 ms, 128 B 1.360 ms; the gather's extra sectors cost no time, so the default leaves it.
static void apply_l2_fetch_limit()
{
  static const bool done = [] {
    size_t bytes = 0;
    if (const char* v = std::getenv("OTG_L2_FETCH_BYTES"))
      bytes = size_t(std::atoi(v));
    if (bytes)
      cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, bytes);
    cudaGetLastError();
    return true;
  }();
  (void)done;
}

int build_tree(TreeState& t, const void* entities, u64 n, u32 maxDepth, const void* box, u64 maxElem, int mem, cudaStream_t st)
{
  apply_l2_fetch_limit();
  const bool isBox = t.kind != OTG_KIND_POINTS;
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
  // node links pack the first-child index in 28 bits
  if (n + u64(D) * (n / (maxElem + 1) + 1) + 2 >= (u64(1) << kChildShift))
  {
    set_error("entity count too large for the 28-bit node index of this build");
    return OTG_ERR_NOT_SUPPORTED;
  }
  t.n = n;
  t.D = D;
  t.maxElem = maxElem;
  t.built = false;
  t.countsKnown = false;
  t.image32 = false;
  t.inserted = false;
  t.retired.clear();
  t.trees = 0;
  t.boxGiven = box != nullptr;
  cudaError_t e;
  if ((e = t.err.ensure(sizeof(u32) * 4)))
    return cuda_status(e, "allocating status word");
  cudaMemsetAsync(t.err.p, 0, sizeof(u32) * 4, st);
  // Host entities are copied to the device; device entities are read in place during the build
  // (the caller keeps them alive until the build completes on `st`, as for any stream-ordered call).
  const void* ent = entities;
  const void* pull = nullptr;
  if (n && mem == OTG_MEM_HOST)
  {
    if ((e = t.entities.ensure(esz * W * n)))
      return cuda_status(e, "allocating entity buffer");
    // Pinned host memory that the device can map is read by the bounding-box pass itself, which
    // writes the device copy as it goes (the upload is bound by the host link either way). Other
    // host memory, or a given space box (no bounding-box pass), is copied first.
    cudaPointerAttributes at{};
    const bool mapped = !box && cudaPointerGetAttributes(&at, entities) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer &&
                        (reinterpret_cast<uintptr_t>(at.devicePointer) & 15) == 0;
    cudaGetLastError(); // a pointer unknown to CUDA leaves no error behind
    if (mapped)
      pull = at.devicePointer;
    else if ((e = cudaMemcpyAsync(t.entities.p, entities, esz * W * n, cudaMemcpyHostToDevice, st)))
      return cuda_status(e, "copying entities");
    ent = t.entities.p;
  }
  const void* dbox = nullptr;
  if (box)
  {
    if ((e = t.boxDev.ensure(esz * 6)))
      return cuda_status(e, "allocating box");
    if ((e = cudaMemcpyAsync(t.boxDev.p, box, esz * 6, mem == OTG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st)))
      return cuda_status(e, "copying box");
    dbox = t.boxDev.p;
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
  // a loose box's location can lie one cell outside the grid (3 more key bits), which a 32-bit
  // key would cut off
  t.keys32 = bits + (isBox ? 3 : 0) <= 32;
  int rc;
  if (t.scalar == OTG_SCALAR_F64)
  {
    const double* p = static_cast<const double*>(ent);
    const double* q = static_cast<const double*>(pull);
    if (isBox)
      rc = t.keys32 ? build_impl<double, u32, true>(t, p, dbox, n, st, q) : build_impl<double, u64, true>(t, p, dbox, n, st, q);
    else
      rc = t.keys32 ? build_impl<double, u32, false>(t, p, dbox, n, st, q) : build_impl<double, u64, false>(t, p, dbox, n, st, q);
  }
  else
  {
    const float* p = static_cast<const float*>(ent);
    const float* q = static_cast<const float*>(pull);
    if (isBox)
      rc = t.keys32 ? build_impl<float, u32, true>(t, p, dbox, n, st, q) : build_impl<float, u64, true>(t, p, dbox, n, st, q);
    else
      rc = t.keys32 ? build_impl<float, u32, false>(t, p, dbox, n, st, q) : build_impl<float, u64, false>(t, p, dbox, n, st, q);
  }
  if (rc)
    return rc;
  t.built = true;
  if (mem == OTG_MEM_HOST)
    return finish_build(t, st);
  return OTG_OK;
}


// ---------------------------------------------------------------- forest: many independent trees
// Several trees are built by one launch sequence. Tree t holds the entities [off[t], off[t+1]) of
// one input array, has its own space box (given, or its entities' bounding box), its own max
// depth (given, or EstimateMaxDepth of its size) and therefore its own threshold tables. Per-tree
// work is expressed through the sort's tile table: tile i is tile segTiles[i].y of tree
// segTiles[i].x, and bounding box, key generation and the segmented radix sort run one block per
// tile. Emission is the single-tree emission with per-node trees: node t is the root of tree t.

template<typename T, int W>
__global__ void __launch_bounds__(256) forest_bbox_kernel(const T* __restrict__ ent, const uint2* __restrict__ segTiles, const u64* __restrict__ off,
                                                          typename Ord<T>::U* __restrict__ acc)
{
  using O = Ord<T>;
  using U = typename O::U;
  const uint2 st = segTiles[blockIdx.x];
  const u64 b = off[st.x] + u64(st.y) * kSortTile;
  const u64 e = min(off[st.x + 1], b + kSortTile);
  U mn[3], mx[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    mn[d] = U(~U(0));
    mx[d] = U(0);
  }
  for (u64 i = b + threadIdx.x; i < e; i += blockDim.x)
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      const U lo = O::of(ent[i * W + d]);
      const U hi = O::of(ent[i * W + (W == 6 ? 3 + d : d)]);
      mn[d] = lo < mn[d] ? lo : mn[d];
      mx[d] = hi > mx[d] ? hi : mx[d];
    }
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
      const U a = __shfl_xor_sync(0xffffffffu, mn[d], o);
      const U c = __shfl_xor_sync(0xffffffffu, mx[d], o);
      mn[d] = a < mn[d] ? a : mn[d];
      mx[d] = c > mx[d] ? c : mx[d];
    }
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      atomicMin(&acc[u64(st.x) * 6 + d], mn[d]);
      atomicMax(&acc[u64(st.x) * 6 + 3 + d], mx[d]);
    }
}

template<typename U>
__global__ void forest_bbox_init_kernel(U* acc, u32 trees)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < u64(trees) * 6; i += u64(gridDim.x) * blockDim.x)
    acc[i] = (i % 6) < 3 ? U(~U(0)) : U(0);
}

template<typename T>
__global__ void forest_space_kernel(Space<T>* __restrict__ sp, const typename Ord<T>::U* __restrict__ acc, const T* __restrict__ boxes,
                                    const u32* __restrict__ treeD, u32 trees, int isPoints)
{
  for (u32 t = blockIdx.x * blockDim.x + threadIdx.x; t < trees; t += gridDim.x * blockDim.x)
  {
    Space<T> s;
    make_space(s, acc + u64(t) * 6, boxes ? boxes + u64(t) * 6 : nullptr, treeD[t], isPoints);
    sp[t] = s;
  }
}

// tree holding entry i of a concatenation with offsets off[0..trees]
__device__ __forceinline__ u32 tree_of(const u64* __restrict__ off, u32 trees, u64 i)
{
  u32 lo = 0, hi = trees; // off[lo] <= i < off[hi]
  while (hi - lo > 1)
  {
    const u32 m = (lo + hi) >> 1;
    if (off[m] <= i)
      lo = m;
    else
      hi = m;
  }
  return lo;
}

template<typename T>
__global__ void forest_tables_kernel(const Space<T>* __restrict__ sp, typename Ord<T>::U* __restrict__ tab, const u64* __restrict__ tabOff, u32 trees,
                                     int isBox)
{
  const u64 total = tabOff[trees];
  for (u64 idx = blockIdx.x * u64(blockDim.x) + threadIdx.x; idx < total; idx += u64(gridDim.x) * blockDim.x)
  {
    const u32 t = tree_of(tabOff, trees, idx);
    const Space<T>& s = sp[t];
    const u32 cells = isBox ? (1u << s.D) + 2 : (1u << s.D);
    const u64 perDim = RasterLayout<T>::per_dim(cells);
    const u64 local = idx - tabOff[t];
    const int d = int(local / perDim);
    const u32 j = u32(local % perDim);
    tab[idx] = s.rasterDouble ? raster_threshold<T, double>(s, d, j, cells, isBox) : raster_threshold<T, float>(s, d, j, cells, isBox);
  }
}

template<typename T>
__global__ void forest_min_table_kernel(const Space<T>* __restrict__ sp, T* __restrict__ tab, const u64* __restrict__ minOff, u32 trees)
{
  const u64 total = minOff[trees];
  for (u64 idx = blockIdx.x * u64(blockDim.x) + threadIdx.x; idx < total; idx += u64(gridDim.x) * blockDim.x)
  {
    const u32 t = tree_of(minOff, trees, idx);
    const Space<T>& s = sp[t];
    const u64 perDim = (u64(2) << s.D) - 1;
    const u64 local = idx - minOff[t];
    tab[idx] = s.rasterDouble ? node_min_entry<T, double>(s, int(local / perDim), local % perDim)
                              : node_min_entry<T, float>(s, int(local / perDim), local % perDim);
  }
}

// One block per sort tile: keys of the tile's entities with its tree's tables (in shared memory
// when they fit), and the tree's radix digit counts ([pass][tree][256]).
template<typename T, typename K, bool IS_BOX>
__global__ void __launch_bounds__(256) forest_codegen_kernel(const T* __restrict__ ent, const uint2* __restrict__ segTiles, const u64* __restrict__ off,
                                                             const Space<T>* __restrict__ sp, const typename Ord<T>::U* __restrict__ tabG,
                                                             const u64* __restrict__ tabOff, int tabInSmem, K* __restrict__ keys, u32* __restrict__ hist,
                                                             u32 trees, u32 passes, bool regular, u32* __restrict__ err)
{
  using U = typename Ord<T>::U;
  constexpr int W = IS_BOX ? 6 : 3;
  extern __shared__ __align__(16) unsigned char s_dyn[];
  __shared__ u32 sh[8][kRadix];
  __shared__ float minF[3], rastF[3], margF[3];
  const uint2 st = segTiles[blockIdx.x];
  const u32 tr = st.x;
  const Space<T>& s = sp[tr];
  const u32 D = s.D;
  const u32 cells = IS_BOX ? (1u << D) + 2 : (1u << D);
  const size_t perDim = RasterLayout<T>::per_dim(cells);
  const U* tab = tabG + tabOff[tr];
  U* stab = reinterpret_cast<U*>(s_dyn);
  for (int i = threadIdx.x; i < 8 * kRadix; i += blockDim.x)
    (&sh[0][0])[i] = 0;
  if (tabInSmem)
    for (size_t i = threadIdx.x; i < 3 * perDim; i += blockDim.x)
      stab[i] = tab[i];
  if (threadIdx.x < 3)
  {
    minF[threadIdx.x] = to_f(s.min[threadIdx.x]);
    rastF[threadIdx.x] = s.rasterDouble ? float(s.rastD[threadIdx.x]) : s.rastF[threadIdx.x];
    margF[threadIdx.x] =
      cell_estimate_margin(s, threadIdx.x, s.rasterDouble ? s.rastD[threadIdx.x] : double(s.rastF[threadIdx.x]), cells);
  }
  __syncthreads();
  if (tabInSmem)
    tab = stab;
  const u64 b = off[tr] + u64(st.y) * kSortTile;
  const u64 e = min(off[tr + 1], b + kSortTile);
  for (u64 i = b + threadIdx.x; i < e; i += blockDim.x)
  {
    T v[W];
#pragma unroll
    for (int c = 0; c < W; ++c)
      v[c] = ent[i * W + c];
    K kk;
    if constexpr (IS_BOX)
    {
      u64 k64 = regular ? regular_box_key<T>(v, s, D) : entity_key<T, IS_BOX>(v, tab, perDim, cells, minF, rastF, D);
      if (k64 == kBadRegularBox)
      {
        atomicOr(err, kErrArgument);
        k64 = 0;
      }
      kk = K(k64);
    }
    else
      kk = K(entity_key<T, IS_BOX, sizeof(K) == 4>(v, tab, perDim, cells, minF, rastF, D, margF));
    keys[i] = kk;
    for (u32 p = 0; p < passes; ++p)
      atomicAdd(&sh[p][(kk >> (kRadixBits * p)) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  for (u32 p = 0; p < passes; ++p)
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
      if (sh[p][d])
        atomicAdd(&hist[(u64(p) * trees + tr) * kRadix + d], sh[p][d]);
}

__global__ void forest_root_init_kernel(uint4* link, u64* nodeKey, unsigned char* nodeDepth, u32* levelCount, const u64* __restrict__ off, u32 trees,
                                        u32* nodeParent, u32* nodeTree)
{
  for (u32 t = blockIdx.x * blockDim.x + threadIdx.x; t < trees; t += gridDim.x * blockDim.x)
  {
    link[t] = make_uint4(0, u32(off[t]), u32(off[t]), u32(off[t + 1]));
    nodeKey[t] = 1;
    nodeDepth[t] = 0;
    nodeTree[t] = t;
    if (nodeParent)
      nodeParent[t] = t;
    if (t == 0)
      levelCount[0] = trees;
  }
}

// launchOnly: the buffers and the host-computed layout of this forest are in place from an earlier
// build with the same tree sizes; only device work is issued (stream-capturable).
template<typename T, typename K, bool IS_BOX>
static int forest_build_impl(TreeState& t, const T* ent, const T* boxes, cudaStream_t st, bool launchOnly = false)
{
  constexpr int W = IS_BOX ? 6 : 3;
  using U = typename Ord<T>::U;
  const bool regular = t.kind == OTG_KIND_BOXES_REGULAR;
  const u32 trees = t.trees;
  const u64 n = t.n;
  const u32 Dmax = t.D;
  // sorted key bits (out-of-grid loose-box locations: three bits above 3D + 5)
  const u32 bits = IS_BOX ? std::min(3 * Dmax + 8, u32(8 * sizeof(K))) : 3 * Dmax + 1;
  const u32 passes = (bits + kRadixBits - 1) / kRadixBits;
  const u32 tiles = u32(t.segTilesHost.size());
  const u64 tabEntries = t.tabOffHost.back();
  const u64 minEntries = IS_BOX ? 1 : t.minOffHost.back();
  u64 maxTab = 0;
  for (u32 i = 0; i < trees; ++i)
    maxTab = std::max(maxTab, t.tabOffHost[i + 1] - t.tabOffHost[i]);
  const size_t maxTabBytes = sizeof(U) * maxTab;
  const u64 maxNodes = n + trees + u64(Dmax) * (n / (t.maxElem + 1) + 1) + 2;
  t.maxNodes = maxNodes;
  const size_t histWords = size_t(passes) * trees * kRadix;
  const size_t scratchWords = histWords + size_t(passes) * std::max<u32>(tiles, 1) * kRadix + passes + 8;
  cudaError_t e;
  if (!launchOnly)
  {
  if ((e = t.keysA.ensure(sizeof(K) * std::max<u64>(n, 1))) || (e = t.keysB.ensure(sizeof(K) * std::max<u64>(n, 1))) ||
      (e = t.sortedIds.ensure(sizeof(u32) * std::max<u64>(n, 1))) || (e = t.valsB.ensure(sizeof(u32) * std::max<u64>(n, 1))) ||
      (e = t.sortedGeom.ensure(sizeof(T) * W * std::max<u64>(n, 1))) || (e = t.nodeLink.ensure(sizeof(uint4) * maxNodes)) ||
      (e = t.nodeKey.ensure(sizeof(u64) * maxNodes)) || (e = t.nodeBox.ensure(sizeof(T) * 6 * maxNodes)) || (e = t.nodeDepth.ensure(maxNodes)) ||
      (e = t.nodeTree.ensure(sizeof(u32) * maxNodes)) || (e = t.levelCount.ensure(sizeof(u32) * 64)) ||
      (e = t.splitQueue.ensure(2 * sizeof(u32) * (n / (t.maxElem + 1) + 2))) || (e = t.space.ensure(sizeof(Space<T>) * trees)) ||
      (e = t.sortScratch.ensure(sizeof(u32) * scratchWords)) || (e = t.bboxBits.ensure(sizeof(U) * 6 * trees)) ||
      (e = t.rasterTab.ensure(sizeof(U) * std::max<u64>(tabEntries, 1))) || (e = t.minTab.ensure(sizeof(T) * minEntries)) ||
      (e = t.treeOff.ensure(sizeof(u64) * (trees + 1))) || (e = t.treeD.ensure(sizeof(u32) * trees)) ||
      (e = t.tabOff.ensure(sizeof(u64) * (trees + 1))) || (e = t.minOff.ensure(sizeof(u64) * (trees + 1))) ||
      (e = t.segTiles.ensure(sizeof(uint2) * std::max<u32>(tiles, 1))) ||
      (IS_BOX && ((e = t.nodeMax.ensure(sizeof(T) * 3 * maxNodes)) || (e = t.ownerNode.ensure(sizeof(u32) * std::max<u64>(n, 1))) ||
                  (e = t.nodeParent.ensure(sizeof(u32) * maxNodes)))))
    return cuda_status(e, "allocating forest buffers");

  // host-computed layout: tree offsets, depths, table offsets, tile table
  cudaMemcpyAsync(t.treeOff.p, t.treeOffHost.data(), sizeof(u64) * (trees + 1), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(t.treeD.p, t.treeDHost.data(), sizeof(u32) * trees, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(t.tabOff.p, t.tabOffHost.data(), sizeof(u64) * (trees + 1), cudaMemcpyHostToDevice, st);
  if (!IS_BOX)
    cudaMemcpyAsync(t.minOff.p, t.minOffHost.data(), sizeof(u64) * (trees + 1), cudaMemcpyHostToDevice, st);
  if (tiles)
    cudaMemcpyAsync(t.segTiles.p, t.segTilesHost.data(), sizeof(uint2) * tiles, cudaMemcpyHostToDevice, st);
  }
  cudaMemsetAsync(t.sortScratch.p, 0, sizeof(u32) * scratchWords, st);
  cudaMemsetAsync(t.levelCount.p, 0, sizeof(u32) * 64, st);
  cudaMemsetAsync(t.err.p, 0, sizeof(u32) * 4, st);

  Profiler idle;
  Profiler& prof = launchOnly ? idle : profiler();
  prof.reset();
  const u64* off = t.treeOff.as<u64>();
  const uint2* segTiles = t.segTiles.as<uint2>();
  Space<T>* sp = t.space.as<Space<T>>();
  prof.mark("bbox", st);
  if (!boxes)
  {
    forest_bbox_init_kernel<U><<<grid_blocks(u64(trees) * 6), 256, 0, st>>>(t.bboxBits.as<U>(), trees);
    if (tiles)
      forest_bbox_kernel<T, W><<<tiles, 256, 0, st>>>(ent, segTiles, off, t.bboxBits.as<U>());
  }
  prof.mark("tables", st);
  forest_space_kernel<T><<<grid_blocks(trees, 128), 128, 0, st>>>(sp, t.bboxBits.as<U>(), boxes, t.treeD.as<u32>(), trees, IS_BOX ? 0 : 1);
  forest_tables_kernel<T><<<grid_blocks(tabEntries, 128, 152 * 32), 128, 0, st>>>(sp, t.rasterTab.as<U>(), t.tabOff.as<u64>(), trees, IS_BOX ? 1 : 0);
  if (!IS_BOX)
    forest_min_table_kernel<T><<<grid_blocks(minEntries), 256, 0, st>>>(sp, t.minTab.as<T>(), t.minOff.as<u64>(), trees);

  prof.mark("codegen", st);
  u32* scratch = t.sortScratch.as<u32>();
  u32* hist = scratch;
  u32* status = scratch + histWords;
  u32* counters = status + size_t(passes) * std::max<u32>(tiles, 1) * kRadix;
  const int tabInSmem = maxTabBytes <= 64 * 1024 ? 1 : 0;
  const size_t cgSmem = tabInSmem ? maxTabBytes : 0;
  if (tiles)
  {
    auto kfn = forest_codegen_kernel<T, K, IS_BOX>;
    cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(cgSmem));
    kfn<<<tiles, 256, cgSmem, st>>>(ent, segTiles, off, sp, t.rasterTab.as<U>(), t.tabOff.as<u64>(), tabInSmem, t.keysA.as<K>(), hist, trees, passes,
                                    regular, t.err.as<u32>());
  }

  prof.mark("sort", st);
  const bool inB = onesweep_passes_segmented<K>(t.keysA.as<K>(), t.sortedIds.as<u32>(), t.keysB.as<K>(), t.valsB.as<u32>(), n, passes, true, segTiles,
                                                tiles, off, trees, hist, status, counters, t.err.as<u32>(), st);
  if (inB)
  {
    std::swap(t.sortedIds, t.valsB);
    t.sortedKeys = t.keysB.p;
  }
  else
    t.sortedKeys = t.keysA.p;
  const K* keys = reinterpret_cast<const K*>(t.sortedKeys);

  // gather, then emission, on one stream: a forest's gather needs the whole GPU (an emission stream
  // beside it measured 1.642 ms against 1.65 ms in sequence for 65.8M boxes, and 1.718 ms with the
  // single tree's thinner gather), so the recorded step keeps a single stream
  const cudaStream_t es = st;
  prof.mark("gather", st);
  if (n)
    gather_kernel<T, W, kGatherPerThread><<<grid_blocks((n + kGatherPerThread - 1) / kGatherPerThread, 256, 152 * 16), 256, 0, st>>>(
      ent, t.sortedIds.as<u32>(), n, t.sortedGeom.as<T>());
  prof.mark("emit", st);
  u32* parent = IS_BOX ? t.nodeParent.as<u32>() : nullptr;
  // entities that the emission places in no node keep kNoOwner
  if (IS_BOX && n)
    if (cudaError_t me = cudaMemsetAsync(t.ownerNode.p, 0xff, sizeof(u32) * n, st))
      return cuda_status(me, "clearing the entity owners");
  forest_root_init_kernel<<<grid_blocks(trees, 128), 128, 0, es>>>(t.nodeLink.as<uint4>(), t.nodeKey.as<u64>(), t.nodeDepth.as<unsigned char>(),
                                                                   t.levelCount.as<u32>(), off, trees, parent, t.nodeTree.as<u32>());
  const int emitBlocks = grid_blocks(maxNodes, 256, 152 * 16);
  u32* levelCount = t.levelCount.as<u32>();
  u32* splitCount = levelCount + 32;
  const u32 queueCap = u32(n / (t.maxElem + 1) + 2);
  const ForestNodes fn{ t.nodeTree.as<u32>(), t.treeD.as<u32>(), IS_BOX ? nullptr : t.minOff.as<u64>() };
  u32* splitQueue = t.splitQueue.as<u32>();
  // the roots' decisions, then one launch per depth (queues of depths d and d + 1 alternate halves)
  emit_classify_kernel<T, IS_BOX><<<emit_blocks(0, trees, emitBlocks, ~u64(0), 256), 256, 0, es>>>(0, Dmax, t.maxElem, t.nodeLink.as<uint4>(),
                                                                                                t.nodeKey.as<u64>(), t.nodeBox.as<T>(), levelCount,
                                                                                                splitCount, splitQueue, queueCap, t.minTab.as<T>(), sp,
                                                                                                IS_BOX ? t.ownerNode.as<u32>() : nullptr,
                                                                                                t.err.as<u32>(), fn);
  for (u32 d = 0; d < Dmax; ++d)
    emit_split_kernel<T, K, IS_BOX><<<emit_blocks(d, trees, emitBlocks, queueCap, 32), 256, 0, es>>>(
      d, Dmax, keys, t.nodeLink.as<uint4>(), t.nodeKey.as<u64>(), t.nodeBox.as<T>(), t.nodeDepth.as<unsigned char>(), levelCount, splitCount,
      splitQueue + (d & 1) * queueCap, queueCap, t.minTab.as<T>(), sp, maxNodes, t.err.as<u32>(), IS_BOX ? t.ownerNode.as<u32>() : nullptr, parent, fn,
      t.maxElem, splitQueue + ((d + 1) & 1) * queueCap);
  prof.mark("geometry", st);
  if constexpr (IS_BOX)
  {
    for (int d = int(Dmax); d >= 0; --d)
      mbr_level_kernel<T><<<emit_blocks(u32(d), trees, emitBlocks, ~u64(0), 256), 256, 0, st>>>(u32(d), levelCount, t.nodeLink.as<uint4>(), t.sortedGeom.as<T>(), t.nodeBox.as<T>(),
                                                      t.nodeMax.as<T>());
  }
  else if (boxes)
    root_box_kernel<T><<<trees, 256, 0, st>>>(t.nodeLink.as<uint4>(), t.sortedGeom.as<T>(), t.nodeBox.as<T>(), sp);
  prof.mark("end", st);
  return cuda_status(cudaGetLastError(), "launching forest build kernels");
}

int build_forest(TreeState& t, const void* entities, const u64* treeOffsets, u32 trees, u32 maxDepth, const void* boxes, u64 maxElem, int mem,
                 cudaStream_t st)
{
  const bool isBox = t.kind != OTG_KIND_POINTS;
  const int W = isBox ? 6 : 3;
  const size_t esz = t.scalar == OTG_SCALAR_F64 ? 8 : 4;
  if (maxElem == 0 || trees == 0 || !treeOffsets || treeOffsets[0] != 0)
  {
    set_error("a forest needs at least one tree, offsets starting at 0 and maxElementNo > 0");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  const u64 n = treeOffsets[trees];
  if (n >= (u64(1) << 30))
  {
    set_error("entity count must be below 2^30");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (maxDepth > 19)
  {
    set_error("maxDepthID must be in [1, 19]");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  t.treeOffHost.assign(treeOffsets, treeOffsets + trees + 1);
  t.treeDHost.resize(trees);
  t.tabOffHost.assign(trees + 1, 0);
  t.minOffHost.assign(trees + 1, 0);
  t.segTilesHost.clear();
  u32 Dmax = 1;
  for (u32 i = 0; i < trees; ++i)
  {
    if (treeOffsets[i + 1] < treeOffsets[i])
    {
      set_error("tree offsets must not decrease");
      return OTG_ERR_INVALID_ARGUMENT;
    }
    const u64 ni = treeOffsets[i + 1] - treeOffsets[i];
    const u32 D = maxDepth ? maxDepth : estimate_max_depth(ni, maxElem);
    t.treeDHost[i] = D;
    Dmax = std::max(Dmax, D);
    const u32 cells = isBox ? (1u << D) + 2 : (1u << D);
    t.tabOffHost[i + 1] = t.tabOffHost[i] + 3 * (2 + kLevelThresholds + cells);
    t.minOffHost[i + 1] = t.minOffHost[i] + 3 * ((u64(2) << D) - 1);
    const u64 nt = (ni + kSortTile - 1) / kSortTile;
    for (u64 k = 0; k < nt; ++k)
      t.segTilesHost.push_back(make_uint2(i, u32(k)));
  }
  if (n + trees + u64(Dmax) * (n / (maxElem + 1) + 1) + 2 >= (u64(1) << kChildShift))
  {
    set_error("entity count too large for the 28-bit node index of this build");
    return OTG_ERR_NOT_SUPPORTED;
  }
  t.n = n;
  t.D = Dmax;
  t.maxElem = maxElem;
  t.built = false;
  t.countsKnown = false;
  t.image32 = false;
  t.inserted = false;
  t.retired.clear();
  t.trees = trees;
  t.boxGiven = boxes != nullptr;
  cudaError_t e;
  if ((e = t.err.ensure(sizeof(u32) * 4)))
    return cuda_status(e, "allocating status word");
  cudaMemsetAsync(t.err.p, 0, sizeof(u32) * 4, st);
  const void* ent = entities;
  if (n && mem == OTG_MEM_HOST)
  {
    if ((e = t.entities.ensure(esz * W * n)))
      return cuda_status(e, "allocating entity buffer");
    if ((e = cudaMemcpyAsync(t.entities.p, entities, esz * W * n, cudaMemcpyHostToDevice, st)))
      return cuda_status(e, "copying entities");
    ent = t.entities.p;
  }
  const void* dboxes = nullptr;
  if (boxes)
  {
    if ((e = t.boxDev.ensure(esz * 6 * trees)))
      return cuda_status(e, "allocating boxes");
    if ((e = cudaMemcpyAsync(t.boxDev.p, boxes, esz * 6 * trees, mem == OTG_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st)))
      return cuda_status(e, "copying boxes");
    dboxes = t.boxDev.p;
  }
  const u32 bits = isBox ? 3 * Dmax + 5 : 3 * Dmax + 1;
  t.keys32 = bits + (isBox ? 3 : 0) <= 32; // out-of-grid loose-box locations need 3 more bits
  int rc;
  if (t.scalar == OTG_SCALAR_F64)
  {
    const double* p = static_cast<const double*>(ent);
    const double* b = static_cast<const double*>(dboxes);
    if (isBox)
      rc = t.keys32 ? forest_build_impl<double, u32, true>(t, p, b, st) : forest_build_impl<double, u64, true>(t, p, b, st);
    else
      rc = t.keys32 ? forest_build_impl<double, u32, false>(t, p, b, st) : forest_build_impl<double, u64, false>(t, p, b, st);
  }
  else
  {
    const float* p = static_cast<const float*>(ent);
    const float* b = static_cast<const float*>(dboxes);
    if (isBox)
      rc = t.keys32 ? forest_build_impl<float, u32, true>(t, p, b, st) : forest_build_impl<float, u64, true>(t, p, b, st);
    else
      rc = t.keys32 ? forest_build_impl<float, u32, false>(t, p, b, st) : forest_build_impl<float, u64, false>(t, p, b, st);
  }
  if (rc)
    return rc;
  t.built = true;
  if (mem == OTG_MEM_HOST)
    return finish_build(t, st);
  return OTG_OK;
}

// Re-issues the device work of the forest's last build on new entity values (same tree sizes,
// depths and boxes); allocates and copies nothing from the host, so it can be stream-captured.
int forest_relaunch(TreeState& t, const void* entities, const void* boxes, cudaStream_t st)
{
  if (!t.trees || !t.built)
  {
    set_error("forest_relaunch needs a forest that was built before");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  const bool isBox = t.kind != OTG_KIND_POINTS;
  int rc;
  if (t.scalar == OTG_SCALAR_F64)
  {
    const double* p = static_cast<const double*>(entities);
    const double* b = static_cast<const double*>(boxes);
    if (isBox)
      rc = t.keys32 ? forest_build_impl<double, u32, true>(t, p, b, st, true) : forest_build_impl<double, u64, true>(t, p, b, st, true);
    else
      rc = t.keys32 ? forest_build_impl<double, u32, false>(t, p, b, st, true) : forest_build_impl<double, u64, false>(t, p, b, st, true);
  }
  else
  {
    const float* p = static_cast<const float*>(entities);
    const float* b = static_cast<const float*>(boxes);
    if (isBox)
      rc = t.keys32 ? forest_build_impl<float, u32, true>(t, p, b, st, true) : forest_build_impl<float, u64, true>(t, p, b, st, true);
    else
      rc = t.keys32 ? forest_build_impl<float, u32, false>(t, p, b, st, true) : forest_build_impl<float, u64, false>(t, p, b, st, true);
  }
  return rc;
}

int finish_build(TreeState& t, cudaStream_t st)
{
  if (t.countsKnown)
    return OTG_OK;
  u32 hostErr = 0;
  std::vector<u32> lc(32, 0);
  cudaError_t e = cudaMemcpyAsync(&hostErr, t.err.p, sizeof(u32), cudaMemcpyDeviceToHost, st);
  if (!e && (t.n || t.trees))
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
  if (hostErr & kErrArgument)
  {
    set_error("a box of a regular box tree has its min corner on the max face of the space, where the reference asserts "
              "(detail/si_grid.h:213)");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (t.n || t.trees)
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

// The Core form's entity span (otg_tree_set_entities): the new geometry in tree order, gathered by
// the ids of the last Create; nodes, node boxes and MBRs stay as that Create built them.
int set_entities(TreeState& t, const void* entities, u64 n, int mem, cudaStream_t st)
{
  if (t.trees)
  {
    set_error("otg_tree_set_entities: not for forests");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (n != t.n)
  {
    set_error("otg_tree_set_entities: the entity count differs from the tree's");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (n == 0)
    return OTG_OK;
  const bool isBox = t.kind != OTG_KIND_POINTS;
  const int W = isBox ? 6 : 3;
  const size_t esz = t.scalar == OTG_SCALAR_F64 ? 8 : 4;
  cudaError_t e;
  const void* src = entities;
  if (mem == OTG_MEM_HOST)
  {
    if ((e = t.entities.ensure(esz * W * n)) || (e = cudaMemcpyAsync(t.entities.p, entities, esz * W * n, cudaMemcpyHostToDevice, st)))
      return cuda_status(e, "copying entities");
    src = t.entities.p;
  }
  const int blocks = grid_blocks((n + kGatherPerThread - 1) / kGatherPerThread, 256, 152 * 16);
  if (t.scalar == OTG_SCALAR_F64)
  {
    if (isBox)
      gather_kernel<double, 6, kGatherPerThread><<<blocks, 256, 0, st>>>((const double*)src, t.sortedIds.as<u32>(), n, t.sortedGeom.as<double>());
    else
      gather_kernel<double, 3, kGatherPerThread><<<blocks, 256, 0, st>>>((const double*)src, t.sortedIds.as<u32>(), n, t.sortedGeom.as<double>());
  }
  else
  {
    if (isBox)
      gather_kernel<float, 6, kGatherPerThread><<<blocks, 256, 0, st>>>((const float*)src, t.sortedIds.as<u32>(), n, t.sortedGeom.as<float>());
    else
      gather_kernel<float, 3, kGatherPerThread><<<blocks, 256, 0, st>>>((const float*)src, t.sortedIds.as<u32>(), n, t.sortedGeom.as<float>());
  }
  t.image32 = false; // the FP32 filter images follow the geometry
  if ((e = cudaGetLastError()))
    return cuda_status(e, "gathering entities");
  if (mem == OTG_MEM_HOST && (e = cudaStreamSynchronize(st)))
    return cuda_status(e, "gathering entities");
  return OTG_OK;
}

int export_locations(const TreeState& t, u64* keys, int mem, cudaStream_t st)
{
  if (t.trees)
  {
    set_error("location export is defined for a single tree, not a forest");
    return OTG_ERR_NOT_SUPPORTED;
  }
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
  const bool isBox = t.kind != OTG_KIND_POINTS;
  const bool rd = t.scalar == OTG_SCALAR_F64 || t.D >= 16;
  const int blocks = grid_blocks(t.n);
  const u32* ids = t.sortedIds.as<u32>();
  if (t.scalar == OTG_SCALAR_F64)
  {
    auto sp = t.space.as<Space<double>>();
    const double* g = t.sortedGeom.as<double>();
    if (isBox)
      location_export_kernel<double, double, true><<<blocks, 256, 0, st>>>(g, ids, t.n, sp, out, t.kind == OTG_KIND_BOXES_REGULAR);
    else
      location_export_kernel<double, double, false><<<blocks, 256, 0, st>>>(g, ids, t.n, sp, out, t.kind == OTG_KIND_BOXES_REGULAR);
  }
  else
  {
    auto sp = t.space.as<Space<float>>();
    const float* g = t.sortedGeom.as<float>();
    if (isBox)
    {
      if (rd)
        location_export_kernel<float, double, true><<<blocks, 256, 0, st>>>(g, ids, t.n, sp, out, t.kind == OTG_KIND_BOXES_REGULAR);
      else
        location_export_kernel<float, float, true><<<blocks, 256, 0, st>>>(g, ids, t.n, sp, out, t.kind == OTG_KIND_BOXES_REGULAR);
    }
    else
    {
      if (rd)
        location_export_kernel<float, double, false><<<blocks, 256, 0, st>>>(g, ids, t.n, sp, out, t.kind == OTG_KIND_BOXES_REGULAR);
      else
        location_export_kernel<float, float, false><<<blocks, 256, 0, st>>>(g, ids, t.n, sp, out, t.kind == OTG_KIND_BOXES_REGULAR);
    }
  }
  cudaError_t e = cudaGetLastError();
  if (!e && mem == OTG_MEM_HOST)
  {
    e = cudaMemcpyAsync(keys, out, sizeof(u64) * t.n, cudaMemcpyDeviceToHost, st);
    if (!e)
      e = cudaStreamSynchronize(st);
  }
  return cuda_status(e, "exporting locations");
}

int export_nodes(const TreeState& t, u64* keys, double* minSize, u64* eoff, u32* eids, u32* childCount)
{
  const u64 m = t.nodeCount;
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
  std::vector<uint4> link(m);
  std::vector<u32> ids(t.n);
  cudaError_t e = cudaMemcpy(link.data(), t.nodeLink.p, sizeof(uint4) * m, cudaMemcpyDeviceToHost);
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

// ================================================================ bulk Insert (point trees)
// Insert(newEntities, existingEntities) of DynamicHashOrthoTreeCore (core/ot_dynamic_hash_core.h:
// 1012-1333) and LinkOrphanNodes (:826-863) for point trees; MinPoint trees need no geometry
// update (UpdateNodeGeometry :866-1005 only unites MBRs). New entity i gets id n + i.
//  1. keys of the new points from the tree's own grid (the rasterisation tables of its Create), and
//     a stable radix sort of them;
//  2. the reference's clustering of the sorted new points, in rounds: an item of at most
//     maxElementNo points becomes one cluster at its location (:1304-1308), an item of at most 256
//     (or one whose remaining bits are 0: identical locations) is walked greedily (:1237-1291, one
//     lane), a larger one is split by the next 9 bits into buckets found by binary search, each with
//     the fold of its locations (lowest common ancestor, :1153-1199). Items and clusters partition
//     the sorted points, so each is stored at the sorted position where it begins: no counters, and
//     a fixed number of rounds (every split takes at least min(9, bits) bits off an item);
//  3. the node set after LinkOrphanNodes: the old nodes, the clusters' nodes and the lowest common
//     ancestors of depth-first neighbours (the branch nodes the linking creates where two nodes
//     claim one child slot); each node's parent is its nearest ancestor in the set (a child link
//     may skip levels);
//  4. the tree laid out again: nodes breadth first by link level (children contiguous, in slot
//     order), entities ordered by their node in depth-first order (own entities and subtrees
//     contiguous, old entities before new ones in a node), MinPoint geometry from the node keys.
// A new point outside the tree's space is refused (OTG_ERR_INVALID_ARGUMENT, nothing inserted): the
// reference would store it with a location code of 0.
namespace otg
{
namespace
{
struct InsItem // a run [b, e) of sorted new points; e == 0: an empty slot
{
  u32 b, e, bits, depth;
  u64 loc;
};

__device__ __forceinline__ u32 ins_fold_depth(u64 diff, u32 D)
{
  const u32 levels = (u32(64 - __clzll(diff)) + 2u) / 3u;
  return levels >= D ? 0u : D - levels;
}
__device__ __forceinline__ u64 ins_node_key(u64 loc, u32 depth, u32 D) { return (u64(1) << (3 * depth)) | (loc >> (3 * (D - depth))); }
__device__ __forceinline__ u32 ins_key_depth(u64 key) { return u32(63 - __clzll(key)) / 3u; }
// depth-first (pre-order) sort key of a node: its location left-aligned to the max depth, then depth
__device__ __forceinline__ u64 ins_dfs_key(u64 key, u32 D)
{
  const u32 d = ins_key_depth(key);
  return (((key ^ (u64(1) << (3 * d))) << (3 * (D - d))) << 5) | d;
}
__device__ __forceinline__ u64 ins_key_of_dfs(u64 c, u32 D)
{
  const u32 d = u32(c & 31u);
  return (u64(1) << (3 * d)) | ((c >> 5) >> (3 * (D - d)));
}
__device__ __forceinline__ u64 ins_node_lca(u64 a, u64 b) // si_morton.h:307-325
{
  if (a == b)
    return a;
  const u32 da = ins_key_depth(a), db = ins_key_depth(b);
  if (da > db)
    a >>= 3 * (da - db);
  else if (db > da)
    b >>= 3 * (db - da);
  const u32 levels = (u32(64 - __clzll(a ^ b)) + 2u) / 3u;
  return a >> (3 * levels);
}
__device__ __forceinline__ u32 ins_lower_bound(const u64* a, u32 lo, u32 hi, u64 v)
{
  while (lo < hi)
  {
    const u32 mid = lo + ((hi - lo) >> 1);
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}
} // namespace

template<typename T, typename R, typename K>
__global__ void __launch_bounds__(256) insert_keys_kernel(const T* __restrict__ pts, u64 n2, const Space<T>* __restrict__ spg,
                                                          const typename Ord<T>::U* __restrict__ tab, u32 cells, K* __restrict__ keys, u32* __restrict__ vals,
                                                          u32* __restrict__ err)
{
  const Space<T>& s = *spg;
  __shared__ float minF[3], rastF[3], margF[3];
  if (threadIdx.x < 3)
  {
    const int d = threadIdx.x;
    minF[d] = to_f(s.min[d]);
    rastF[d] = float(Raster<R, T>::rast(s, d));
    margF[d] = cell_estimate_margin(s, d, double(Raster<R, T>::rast(s, d)), cells);
  }
  __syncthreads();
  const size_t perDim = RasterLayout<T>::per_dim(cells);
  const u32 D = s.D;
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n2; i += u64(gridDim.x) * blockDim.x)
  {
    const T e[3] = { pts[3 * i], pts[3 * i + 1], pts[3 * i + 2] };
    const u64 k = entity_key<T, false>(e, tab, perDim, cells, minF, rastF, D, margF);
    if (k == 0)
      atomicOr(err, kErrArgument); // outside the space
    keys[i] = K(k);
    vals[i] = u32(i);
  }
}

// One round of the clustering over the item slots `in` (n2 of them, most empty): clusters go to
// (clEnd, clKey) at their first position, items to split to the list `splits` (their buckets are
// searched by insert_split_kernel, one thread per bucket). The 32 slots of a warp are taken in
// turn, each valid one by the whole warp. keys: the sorted new keys (location + 1).
__global__ void __launch_bounds__(256) insert_round_kernel(const u64* __restrict__ keys, u32 n2, u32 D, u64 maxElem, const InsItem* __restrict__ in,
                                                           u32* __restrict__ clEnd, u64* __restrict__ clKey, InsItem* __restrict__ splits,
                                                           u32* __restrict__ nSplits, u32 splitCap, u32* __restrict__ err)
{
  const u32 lane = threadIdx.x & 31;
  const u32 warps = (gridDim.x * blockDim.x) >> 5;
  for (u32 base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32; base < n2; base += warps * 32)
  {
    const u32 p = base + lane;
    InsItem mine{ 0, 0, 0, 0, 0 };
    if (p < n2)
      mine = in[p];
    u32 todo = __ballot_sync(0xffffffffu, mine.e != 0);
    while (todo)
    {
      const int src = __ffs(todo) - 1;
      todo &= todo - 1;
      InsItem w;
      w.b = __shfl_sync(0xffffffffu, mine.b, src);
      w.e = __shfl_sync(0xffffffffu, mine.e, src);
      w.bits = __shfl_sync(0xffffffffu, mine.bits, src);
      w.depth = __shfl_sync(0xffffffffu, mine.depth, src);
      w.loc = __shfl_sync(0xffffffffu, mine.loc, src);
      const u32 num = w.e - w.b;
      if (num <= maxElem) // :1304-1308 one cluster at the item's fold
      {
        if (lane == 0)
        {
          clEnd[w.b] = w.e;
          clKey[w.b] = ins_node_key(w.loc, w.depth, D);
        }
        continue;
      }
      if (w.bits == 0) // identical locations: the walk makes one cluster of them at the max depth
      {
        if (lane == 0)
        {
          clEnd[w.b] = w.e;
          clKey[w.b] = ins_node_key(keys[w.b] - 1, D, D);
        }
        continue;
      }
      if (num <= 256) // :1310-1317 emitSortedRange (:1237-1291), sequential on one lane
      {
        if (lane == 0)
        {
          u32 cb = w.b;
          while (cb < w.e)
          {
            const u64 first = keys[cb] - 1;
            u64 diff = 0;
            u32 ce = cb + 1;
            while (ce < w.e)
            {
              const u64 nd = diff | (first ^ (keys[ce] - 1));
              const u32 newDepth = ins_fold_depth(nd, D);
              if (u64(ce - cb + 1) > maxElem && newDepth < D && newDepth < ins_fold_depth(diff, D))
                break;
              diff = nd;
              ++ce;
            }
            clEnd[cb] = ce;
            clKey[cb] = ins_node_key(first, ins_fold_depth(diff, D), D);
            cb = ce;
          }
        }
        continue;
      }
      // radixPartition (:1153-1199): to the list of items to split
      if (lane == 0)
      {
        const u32 slot = atomicAdd(nSplits, 1u);
        if (slot < splitCap)
          splits[slot] = w;
        else
          atomicOr(err, kErrCapacity);
      }
    }
  }
}

// radixPartition (:1153-1199) of the listed items, one thread per (item, bucket of the next
// min(9, bits) bits): the bucket's run by two binary searches, its fold from its first and last
// location, the child item written to `out` at its first position. All locations of an item share
// the bits above its remaining bits.
__global__ void __launch_bounds__(256) insert_split_kernel(const u64* __restrict__ keys, u32 D, const InsItem* __restrict__ splits,
                                                           const u32* __restrict__ nSplits, u32 splitCap, InsItem* __restrict__ out)
{
  const u64 tasks = u64(min(*nSplits, splitCap)) << 9;
  for (u64 t = blockIdx.x * u64(blockDim.x) + threadIdx.x; t < tasks; t += u64(gridDim.x) * blockDim.x)
  {
    const InsItem w = splits[t >> 9];
    const u32 d = u32(t & 511u);
    const u32 numBits = min(9u, w.bits);
    if (d >= (1u << numBits))
      continue;
    const u32 shift = w.bits - numBits;
    const u64 prefix = w.bits >= 64 ? 0 : (((keys[w.b] - 1) >> w.bits) << w.bits);
    const u64 lo = prefix | (u64(d) << shift);
    const u64 hi = lo + (u64(1) << shift);
    const u32 bb = ins_lower_bound(keys, w.b, w.e, lo + 1);
    const u32 be = ins_lower_bound(keys, bb, w.e, hi + 1);
    if (be > bb)
    {
      const u64 l0 = keys[bb] - 1, l1 = keys[be - 1] - 1;
      const u32 depth = ins_fold_depth(l0 ^ l1, D);
      out[bb] = InsItem{ bb, be, min((D - depth) * 3u, shift), depth, l0 };
    }
  }
}

__global__ void insert_root_item_kernel(InsItem* items, u32 n2, u32 D)
{
  if (blockIdx.x == 0 && threadIdx.x == 0)
    items[0] = InsItem{ 0, n2, 3 * D, 0, 0 };
}

// exclusive scan of u32 values (three launches: block sums, their scan, the adds)
constexpr u32 kScanBlock = 1024;
__global__ void __launch_bounds__(kScanBlock) scan_block_sums_kernel(const u32* __restrict__ v, u32 m, u32* __restrict__ sums)
{
  __shared__ u32 s[32];
  const u32 i = blockIdx.x * kScanBlock + threadIdx.x;
  u32 x = i < m ? v[i] : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0)
    s[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x < 32)
  {
    u32 y = s[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      y += __shfl_xor_sync(0xffffffffu, y, o);
    if (threadIdx.x == 0)
      sums[blockIdx.x] = y;
  }
}
__global__ void __launch_bounds__(kScanBlock) scan_sums_kernel(u32* __restrict__ sums, u32 nb, u32* __restrict__ total)
{
  __shared__ u32 s[32];
  __shared__ u32 carry;
  if (threadIdx.x == 0)
    carry = 0;
  __syncthreads();
  for (u32 base = 0; base < nb; base += kScanBlock)
  {
    const u32 i = base + threadIdx.x;
    const u32 v = i < nb ? sums[i] : 0u;
    u32 x = v;
    const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const u32 y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= u32(o))
        x += y;
    }
    if (lane == 31)
      s[w] = x;
    __syncthreads();
    if (w == 0)
    {
      u32 y = s[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1)
      {
        const u32 z = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= u32(o))
          y += z;
      }
      s[lane] = y;
    }
    __syncthreads();
    const u32 incl = x + (w ? s[w - 1] : 0u);
    if (i < nb)
      sums[i] = carry + incl - v;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1)
      carry += incl;
    __syncthreads();
  }
  if (threadIdx.x == 0)
    *total = carry;
}
__global__ void __launch_bounds__(kScanBlock) scan_add_kernel(const u32* __restrict__ v, u32 m, const u32* __restrict__ sums, u32* __restrict__ out)
{
  __shared__ u32 s[32];
  const u32 i = blockIdx.x * kScanBlock + threadIdx.x;
  const u32 val = i < m ? v[i] : 0u;
  u32 x = val;
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const u32 y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= u32(o))
      x += y;
  }
  if (lane == 31)
    s[w] = x;
  __syncthreads();
  if (w == 0)
  {
    u32 y = s[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const u32 z = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= u32(o))
        y += z;
    }
    s[lane] = y;
  }
  __syncthreads();
  if (i < m)
    out[i] = sums[blockIdx.x] + x - val + (w ? s[w - 1] : 0u);
}

// exclusive scan of v[0, m) into out; *total (device) the sum
static int exclusive_scan_u32(const u32* v, u32 m, u32* out, u32* total, cudaStream_t st)
{
  const u32 nb = std::max<u32>(1, (m + kScanBlock - 1) / kScanBlock);
  TmpBuf sums;
  if (cudaError_t e = sums.ensure(sizeof(u32) * nb, st))
    return cuda_status(e, "allocating scan sums");
  scan_block_sums_kernel<<<nb, kScanBlock, 0, st>>>(v, m, sums.as<u32>());
  scan_sums_kernel<<<1, kScanBlock, 0, st>>>(sums.as<u32>(), nb, total);
  scan_add_kernel<<<nb, kScanBlock, 0, st>>>(v, m, sums.as<u32>(), out);
  return cuda_status(cudaGetLastError(), "scanning");
}

__global__ void insert_cluster_flags_kernel(const u32* __restrict__ clEnd, u32 n2, u32* __restrict__ flag)
{
  for (u32 p = blockIdx.x * blockDim.x + threadIdx.x; p < n2; p += gridDim.x * blockDim.x)
    flag[p] = clEnd[p] != 0 ? 1u : 0u;
}

// node-set entries: old nodes (tag = old index), then clusters (tag = M + cluster), as depth-first
// keys; the clusters are compacted from their slots on the way
__global__ void insert_entries_kernel(const u64* __restrict__ nodeKey, u32 M, const u32* __restrict__ clEnd, const u64* __restrict__ clKey,
                                      const u32* __restrict__ clIdx, u32 n2, u32 D, u64* __restrict__ ek, u32* __restrict__ ev, u32* __restrict__ clBegin)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < M + n2; i += gridDim.x * blockDim.x)
  {
    if (i < M)
    {
      ek[i] = ins_dfs_key(nodeKey[i], D);
      ev[i] = i;
    }
    else if (clEnd[i - M] != 0)
    {
      const u32 p = i - M, c = clIdx[p];
      ek[M + c] = ins_dfs_key(clKey[p], D);
      ev[M + c] = M + c;
      clBegin[c] = p;
    }
  }
}

__global__ void insert_first_kernel(const u64* __restrict__ ek, u32 m, u32* __restrict__ first)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    first[i] = (i == 0 || ek[i] != ek[i - 1]) ? 1u : 0u;
}

// the distinct keys s0 of the sorted entries, and the distinct index of each old node and cluster
__global__ void insert_unique_kernel(const u64* __restrict__ ek, const u32* __restrict__ ev, const u32* __restrict__ first, const u32* __restrict__ idx,
                                     u32 m, u64* __restrict__ s0, u32* __restrict__ s0Of)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
  {
    const u32 u = idx[i] + first[i] - 1;
    if (first[i])
      s0[u] = ek[i];
    s0Of[ev[i]] = u;
  }
}

// the lowest common ancestor of each pair of depth-first neighbours that is missing from s0
// (a neighbour that is an ancestor of the next one gives nothing new)
__global__ void insert_lca_kernel(const u64* __restrict__ s0, u32 U, u32 D, u64* __restrict__ cand, u32* __restrict__ flag)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < U; i += gridDim.x * blockDim.x)
  {
    u32 f = 0;
    if (i > 0)
    {
      const u64 a = ins_key_of_dfs(s0[i - 1], D);
      const u64 l = ins_node_lca(a, ins_key_of_dfs(s0[i], D));
      if (l != a)
      {
        const u64 c = ins_dfs_key(l, D);
        const u32 j = ins_lower_bound(s0, 0, i - 1, c); // an ancestor of s0[i - 1] precedes it
        if (s0[j] != c)
        {
          cand[i] = c;
          f = 1;
        }
      }
    }
    flag[i] = f;
  }
}
__global__ void insert_compact_u64_kernel(const u64* __restrict__ v, const u32* __restrict__ flag, const u32* __restrict__ idx, u32 m, u64* __restrict__ out)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    if (flag[i])
      out[idx[i]] = v[i];
}

// The node set fk = s0 and the new branch nodes nw (sorted, distinct, none in s0), merged: every key
// goes to its index plus the count of the other list's keys below it.
__global__ void insert_place_s0_kernel(const u64* __restrict__ s0, u32 U, const u64* __restrict__ nw, u32 L, u64* __restrict__ fk, u32* __restrict__ map)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < U; i += gridDim.x * blockDim.x)
  {
    const u32 k = i + ins_lower_bound(nw, 0, L, s0[i]);
    fk[k] = s0[i];
    map[i] = k;
  }
}
__global__ void insert_place_new_kernel(const u64* __restrict__ s0, u32 U, const u64* __restrict__ nw, u32 L, u64* __restrict__ fk)
{
  for (u32 q = blockIdx.x * blockDim.x + threadIdx.x; q < L; q += gridDim.x * blockDim.x)
    fk[q + ins_lower_bound(s0, 0, U, nw[q])] = nw[q];
}
// the node index of every old node and every cluster
__global__ void insert_node_index_kernel(const u32* __restrict__ s0Of, const u32* __restrict__ map, u32 M, u32 C, u32* __restrict__ oldToNew,
                                         u32* __restrict__ clusterNode)
{
  for (u32 t = blockIdx.x * blockDim.x + threadIdx.x; t < M + C; t += gridDim.x * blockDim.x)
  {
    const u32 v = map[s0Of[t]];
    if (t < M)
      oldToNew[t] = v;
    else
      clusterNode[t - M] = v;
  }
}

// Parent of every node, nodes in depth-first order (fk sorted, closed under lowest common
// ancestors): the parent of node u > 0 is the lowest common ancestor of nodes u - 1 and u. (Any
// ancestor w of u in the set precedes u, and every node between w and u in depth-first order lies
// in w's subtree; so u - 1 is w or below it, and no set node lies between that ancestor and u.)
// slot: u's child slot in its parent; occupied: the parent's slots as a bit mask; depthCount: nodes
// per depth.
__global__ void insert_parents_kernel(const u64* __restrict__ fk, u32 F, u32 D, u32* __restrict__ parent, unsigned char* __restrict__ slot,
                                      u32* __restrict__ occupied, u32* __restrict__ depthCount, u32* __restrict__ err)
{
  __shared__ u32 sDepth[32]; // nodes per depth of this block, added to depthCount once per block
  if (threadIdx.x < 32)
    sDepth[threadIdx.x] = 0;
  __syncthreads();
  for (u32 u = blockIdx.x * blockDim.x + threadIdx.x; u < F; u += gridDim.x * blockDim.x)
  {
    atomicAdd(&sDepth[u32(fk[u] & 31u)], 1u);
    if (u == 0)
    {
      parent[0] = 0xffffffffu;
      slot[0] = 0;
      continue;
    }
    const u64 key = ins_key_of_dfs(fk[u], D);
    const u64 pk = ins_node_lca(ins_key_of_dfs(fk[u - 1], D), key);
    const u64 pc = ins_dfs_key(pk, D);
    const u32 p = ins_lower_bound(fk, 0, u, pc);
    // a parent missing from the set would be a broken closure: reported, never followed
    if (p >= u || fk[p] != pc || pk == key)
    {
      atomicOr(err, kErrCapacity);
      parent[u] = 0xffffffffu;
      slot[u] = 0;
      continue;
    }
    const u32 s = u32((key >> (3 * (ins_key_depth(key) - ins_key_depth(pk) - 1))) & 7u); // si_morton.h:651-658
    parent[u] = p;
    slot[u] = (unsigned char)s;
    atomicOr(&occupied[p], 1u << s);
  }
  __syncthreads();
  if (threadIdx.x < 32 && sDepth[threadIdx.x])
    atomicAdd(&depthCount[threadIdx.x], sDepth[threadIdx.x]);
}

// Link level (ancestors in the set) of every node by pointer jumping: after round r, lvl[u] counts
// u's ancestors up to (not including) anc[u], its 2^r-th ancestor or the root. Reads one buffer
// pair and writes the other.
__global__ void insert_level_init_kernel(const u32* __restrict__ parent, u32 F, u32* __restrict__ lvl, u32* __restrict__ anc)
{
  for (u32 u = blockIdx.x * blockDim.x + threadIdx.x; u < F; u += gridDim.x * blockDim.x)
  {
    const u32 p = parent[u];
    const bool top = u == 0 || p >= F; // the root (or a node whose parent went missing, reported)
    lvl[u] = top ? 0u : 1u;
    anc[u] = top ? 0u : p;
  }
}
__global__ void insert_level_jump_kernel(const u32* __restrict__ lvl, const u32* __restrict__ anc, u32 F, u32* __restrict__ lvlOut, u32* __restrict__ ancOut)
{
  for (u32 u = blockIdx.x * blockDim.x + threadIdx.x; u < F; u += gridDim.x * blockDim.x)
  {
    const u32 a = anc[u];
    lvlOut[u] = lvl[u] + lvl[a];
    ancOut[u] = anc[a];
  }
}
__global__ void iota_u32_kernel(u32* __restrict__ a, u32 n)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    a[i] = i;
}

// breadth-first position of every node from the stable order by (level, depth-first index), and each
// node's first child: its child of the lowest occupied slot
__global__ void insert_positions_kernel(const u32* __restrict__ bfsToDfs, u32 F, u32* __restrict__ pos)
{
  for (u32 b = blockIdx.x * blockDim.x + threadIdx.x; b < F; b += gridDim.x * blockDim.x)
    pos[bfsToDfs[b]] = b;
}
__global__ void insert_first_child_kernel(const u32* __restrict__ parent, const unsigned char* __restrict__ slot, const u32* __restrict__ occupied,
                                          const u32* __restrict__ pos, u32 F, u32* __restrict__ firstChild)
{
  for (u32 u = 1 + blockIdx.x * blockDim.x + threadIdx.x; u < F; u += gridDim.x * blockDim.x)
  {
    const u32 p = parent[u];
    if (p < F && (occupied[p] & ((1u << slot[u]) - 1u)) == 0)
      firstChild[p] = pos[u];
  }
}

// owner (depth-first node index) of every old entity position, from the old nodes' own ranges; in
// the old order, which is the depth-first order of the old nodes and so non-decreasing
__global__ void insert_old_owner_kernel(const uint4* __restrict__ link, u32 M, u32 n, const u32* __restrict__ oldToNew, u32* __restrict__ owner)
{
  for (u32 j = blockIdx.x * blockDim.x + threadIdx.x; j < M; j += gridDim.x * blockDim.x)
  {
    const uint4 L = link[j];
    for (u32 p = L.y; p < min(L.z, n); ++p)
      owner[p] = oldToNew[j];
  }
}
__global__ void insert_fill_kernel(u32* __restrict__ a, u64 n, u32 v)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
    a[i] = v;
}
// owner of every new entity (sorted position) and its position, for a stable sort by owner
__global__ void insert_new_owner_kernel(const u32* __restrict__ clBegin, const u32* __restrict__ clEnd, u32 C, const u32* __restrict__ clusterNode,
                                        u32* __restrict__ owner, u32* __restrict__ idx)
{
  for (u32 c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x)
  {
    const u32 b = clBegin[c], e = clEnd[b];
    for (u32 p = b; p < e; ++p)
    {
      owner[p] = clusterNode[c];
      idx[p] = p;
    }
  }
}

// start[v] = the first position in owner[0, m) (sorted, below F) whose owner is at least v, for v in
// [0, F]: the change of owner at position k covers the owners it passes
__global__ void insert_starts_kernel(const u32* __restrict__ owner, u64 m, u32 F, u32* __restrict__ start)
{
  for (u64 k = blockIdx.x * u64(blockDim.x) + threadIdx.x; k <= m; k += u64(gridDim.x) * blockDim.x)
  {
    const u32 lo = k == 0 ? 0u : min(owner[k - 1], F) + 1u; // owners up to owner[k - 1] start earlier
    const u32 hi = k == m ? F : min(owner[k], F);           // owners up to owner[k] start here at the latest
    for (u32 v = lo; v <= hi; ++v)
      start[v] = u32(k);
  }
}

// Entities in their new order (by node, old before new within a node): old entity i goes to
// i + (new entities of earlier nodes), new entity j (sorted by node) to j + (old entities of its
// node and earlier ones).
template<typename T>
__global__ void insert_old_entities_kernel(const u32* __restrict__ oldOwner, u32 n, const u32* __restrict__ startNew, const u32* __restrict__ oldIds,
                                           const T* __restrict__ oldGeom, u32* __restrict__ ids, T* __restrict__ geom)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
  {
    const u64 k = u64(i) + startNew[oldOwner[i]];
    ids[k] = oldIds[i];
#pragma unroll
    for (int c = 0; c < 3; ++c)
      geom[k * 3 + c] = oldGeom[u64(i) * 3 + c];
  }
}
template<typename T>
__global__ void insert_new_entities_kernel(const u32* __restrict__ newOwner, const u32* __restrict__ newPos, u32 n2, const u32* __restrict__ startOld,
                                           const u32* __restrict__ newIdx, const T* __restrict__ newPts, u32 n, u32* __restrict__ ids, T* __restrict__ geom)
{
  for (u32 j = blockIdx.x * blockDim.x + threadIdx.x; j < n2; j += gridDim.x * blockDim.x)
  {
    const u64 k = u64(j) + startOld[newOwner[j] + 1];
    const u32 q = newIdx[newPos[j]]; // input index of the new point at sorted position newPos[j]
    ids[k] = n + q;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      geom[k * 3 + c] = newPts[u64(q) * 3 + c];
  }
}

// node records at their positions: links, keys, MinPoint geometry (the root keeps its box)
template<typename T>
__global__ void insert_nodes_kernel(const u32* __restrict__ pos, u32 F, const u64* __restrict__ fk, u32 D, const u32* __restrict__ startOld,
                                    const u32* __restrict__ startNew, const u32* __restrict__ firstChild, const u32* __restrict__ occupied,
                                    const T* __restrict__ oldRootBox, const T* __restrict__ minTab, const Space<T>* __restrict__ spg,
                                    uint4* __restrict__ link, u64* __restrict__ nodeKey, T* __restrict__ nodeBox, unsigned char* __restrict__ nodeDepth)
{
  for (u32 u = blockIdx.x * blockDim.x + threadIdx.x; u < F; u += gridDim.x * blockDim.x)
  {
    const u32 b = pos[u];
    const u64 key = ins_key_of_dfs(fk[u], D);
    const u32 d = ins_key_depth(key);
    // the subtree: the depth-first keys from this node's up to the next cell of its depth
    const u64 loc = key ^ (u64(1) << (3 * d));
    const u64 endKey = ((loc + 1) << (3 * (D - d))) << 5;
    const u32 j = ins_lower_bound(fk, u + 1, F, endKey);
    const u32 cc = __popc(occupied[u]);
    link[b] = make_uint4((cc ? firstChild[u] : 0u) | (cc << kChildShift), startOld[u] + startNew[u], startOld[u + 1] + startNew[u + 1],
                         startOld[j] + startNew[j]);
    nodeKey[b] = key;
    nodeDepth[b] = (unsigned char)d;
    if (b == 0)
    {
#pragma unroll
      for (int c = 0; c < 6; ++c)
        nodeBox[c] = oldRootBox[c];
    }
    else
      write_node_min(nodeBox, b, key, d, minTab, (u64(2) << D) - 1, spg->nodeSize);
  }
}

template<typename T, typename R>
static int insert_impl(TreeState& t, const T* pts, u64 n2, cudaStream_t st)
{
  using U = typename Ord<T>::U;
  const u32 D = t.D;
  const u64 n = t.n;
  const u32 M = u32(t.nodeCount);
  const u64 nt = n + n2;
  u32* err = t.err.as<u32>();
  cudaError_t e;
  u32 hostErr = 0;
  auto read_err = [&](const char* what) -> int {
    cudaError_t ce = cudaMemcpyAsync(&hostErr, err, sizeof(u32), cudaMemcpyDeviceToHost, st);
    if (!ce)
      ce = cudaStreamSynchronize(st);
    if (ce)
      return cuda_status(ce, what);
    return OTG_OK;
  };
  // counts read back by the host: [0] clusters, [1] distinct keys, [2] new branch nodes, [3] spare
  u32* hostCounts = nullptr;
  TmpBuf counts;
  if ((e = counts.ensure(sizeof(u32) * 4, st)))
    return cuda_status(e, "allocating insert counts");
  u32* dCounts = counts.as<u32>();
  u32 hc[4] = { 0, 0, 0, 0 };
  (void)hostCounts;
  auto read_count = [&](int i, const char* what) -> int {
    cudaError_t ce = cudaMemcpyAsync(&hc[i], dCounts + i, sizeof(u32), cudaMemcpyDeviceToHost, st);
    if (!ce)
      ce = cudaStreamSynchronize(st);
    return ce ? cuda_status(ce, what) : OTG_OK;
  };
  Profiler& prof = profiler();
  prof.reset();
  prof.mark("keys", st);
  cudaMemsetAsync(err, 0, sizeof(u32), st);

  // 1. keys of the new points, sorted (stable: equal locations keep their input order)
  TmpBuf nk, nv;
  if ((e = nk.ensure(sizeof(u64) * n2, st)) || (e = nv.ensure(sizeof(u32) * n2, st)))
    return cuda_status(e, "allocating insert keys");
  insert_keys_kernel<T, R, u64><<<blocks_for(n2), 256, 0, st>>>(pts, n2, t.space.as<Space<T>>(), t.rasterTab.as<U>(), 1u << D, nk.as<u64>(),
                                                                nv.as<u32>(), err);
  if (int rc = read_err("computing insert keys"))
    return rc;
  if (hostErr & kErrArgument)
  {
    set_error("otg_tree_insert: a point lies outside the tree's space (nothing inserted)");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (int rc = sort_pairs_u64(nk.as<u64>(), nv.as<u32>(), n2, 3 * D + 1, st, err))
    return rc;

  // 2. clustering rounds over item slots: at most ceil(3D / 9) splits, then the emitting round
  prof.mark("cluster", st);
  TmpBuf itemsA, itemsB, clEnd, clKey, clIdx, splits, nSplits;
  const u32 splitCap = u32(n2 / 257 + 1); // items split in one round hold more than 256 points each
  if ((e = itemsA.ensure(sizeof(InsItem) * n2, st)) || (e = itemsB.ensure(sizeof(InsItem) * n2, st)) || (e = clEnd.ensure(sizeof(u32) * n2, st)) ||
      (e = clKey.ensure(sizeof(u64) * n2, st)) || (e = clIdx.ensure(sizeof(u32) * n2, st)) || (e = splits.ensure(sizeof(InsItem) * splitCap, st)) ||
      (e = nSplits.ensure(sizeof(u32), st)))
    return cuda_status(e, "allocating insert work");
  cudaMemsetAsync(itemsA.p, 0, sizeof(InsItem) * n2, st);
  cudaMemsetAsync(clEnd.p, 0, sizeof(u32) * n2, st);
  insert_root_item_kernel<<<1, 32, 0, st>>>(itemsA.as<InsItem>(), u32(n2), D);
  const u32 rounds = (3 * D + 8) / 9 + 1;
  const int roundBlocks = grid_blocks((n2 + 31) / 32 * 32, 256);
  for (u32 r = 0; r < rounds; ++r)
  {
    cudaMemsetAsync(itemsB.p, 0, sizeof(InsItem) * n2, st);
    cudaMemsetAsync(nSplits.p, 0, sizeof(u32), st);
    insert_round_kernel<<<roundBlocks, 256, 0, st>>>(nk.as<u64>(), u32(n2), D, t.maxElem, itemsA.as<InsItem>(), clEnd.as<u32>(), clKey.as<u64>(),
                                                     splits.as<InsItem>(), nSplits.as<u32>(), splitCap, err);
    insert_split_kernel<<<grid_blocks(u64(splitCap) << 9, 256), 256, 0, st>>>(nk.as<u64>(), D, splits.as<InsItem>(), nSplits.as<u32>(), splitCap,
                                                                             itemsB.as<InsItem>());
    swap(itemsA, itemsB);
  }
  itemsA.release();
  itemsB.release();
  splits.release();
  // cluster c: the c-th occupied slot (a scan of the slot flags)
  if (int rc = [&] {
        TmpBuf flag;
        if (cudaError_t fe = flag.ensure(sizeof(u32) * n2, st))
          return cuda_status(fe, "allocating cluster flags");
        insert_cluster_flags_kernel<<<blocks_for(n2), 256, 0, st>>>(clEnd.as<u32>(), u32(n2), flag.as<u32>());
        return exclusive_scan_u32(flag.as<u32>(), u32(n2), clIdx.as<u32>(), dCounts + 0, st);
      }())
    return rc;
  if (int rc = read_count(0, "clustering inserted points"))
    return rc;
  const u32 C = hc[0];

  // 3. node set: old nodes, cluster nodes and the lowest common ancestors of depth-first neighbours
  prof.mark("node set", st);
  const u64 m = u64(M) + C;
  if (2 * m + 1 >= (u64(1) << kChildShift))
  {
    set_error("otg_tree_insert: node count too large for the 28-bit node index of this build");
    return OTG_ERR_NOT_SUPPORTED;
  }
  const u32 keyBits = 3 * D + 5;
  TmpBuf ek, ev, first, idx, s0, s0Of, clBegin;
  if ((e = ek.ensure(sizeof(u64) * m, st)) || (e = ev.ensure(sizeof(u32) * m, st)) || (e = first.ensure(sizeof(u32) * m, st)) ||
      (e = idx.ensure(sizeof(u32) * m, st)) || (e = s0.ensure(sizeof(u64) * m, st)) || (e = s0Of.ensure(sizeof(u32) * m, st)) ||
      (e = clBegin.ensure(sizeof(u32) * std::max<u32>(C, 1), st)))
    return cuda_status(e, "allocating insert node merge");
  insert_entries_kernel<<<blocks_for(M + n2), 256, 0, st>>>(t.nodeKey.as<u64>(), M, clEnd.as<u32>(), clKey.as<u64>(), clIdx.as<u32>(), u32(n2), D,
                                                            ek.as<u64>(), ev.as<u32>(), clBegin.as<u32>());
  clKey.release();
  clIdx.release();
  if (int rc = sort_pairs_u64(ek.as<u64>(), ev.as<u32>(), m, keyBits, st, err))
    return rc;
  insert_first_kernel<<<blocks_for(m), 256, 0, st>>>(ek.as<u64>(), u32(m), first.as<u32>());
  if (int rc = exclusive_scan_u32(first.as<u32>(), u32(m), idx.as<u32>(), dCounts + 1, st))
    return rc;
  insert_unique_kernel<<<blocks_for(m), 256, 0, st>>>(ek.as<u64>(), ev.as<u32>(), first.as<u32>(), idx.as<u32>(), u32(m), s0.as<u64>(), s0Of.as<u32>());
  if (int rc = read_count(1, "merging insert nodes"))
    return rc;
  const u32 Un = hc[1];
  // branch nodes missing from the set: found per neighbour pair, compacted, sorted, made distinct
  TmpBuf cand, candIdx, nw, nwVals;
  if ((e = cand.ensure(sizeof(u64) * Un, st)) || (e = candIdx.ensure(sizeof(u32) * Un, st)))
    return cuda_status(e, "allocating insert branch nodes");
  insert_lca_kernel<<<blocks_for(Un), 256, 0, st>>>(s0.as<u64>(), Un, D, cand.as<u64>(), first.as<u32>());
  if (int rc = exclusive_scan_u32(first.as<u32>(), Un, candIdx.as<u32>(), dCounts + 2, st))
    return rc;
  if (int rc = read_count(2, "finding insert branch nodes"))
    return rc;
  const u32 L0 = hc[2];
  u32 L = 0;
  if (L0)
  {
    if ((e = nw.ensure(sizeof(u64) * L0, st)) || (e = nwVals.ensure(sizeof(u32) * L0, st)))
      return cuda_status(e, "allocating insert branch nodes");
    insert_compact_u64_kernel<<<blocks_for(Un), 256, 0, st>>>(cand.as<u64>(), first.as<u32>(), candIdx.as<u32>(), Un, nw.as<u64>());
    iota_u32_kernel<<<blocks_for(L0), 256, 0, st>>>(nwVals.as<u32>(), L0);
    if (int rc = sort_pairs_u64(nw.as<u64>(), nwVals.as<u32>(), L0, keyBits, st, err))
      return rc;
    // one node may be the branch of several neighbour pairs: keep each once
    insert_first_kernel<<<blocks_for(L0), 256, 0, st>>>(nw.as<u64>(), L0, first.as<u32>());
    if (int rc = exclusive_scan_u32(first.as<u32>(), L0, candIdx.as<u32>(), dCounts + 3, st))
      return rc;
    insert_compact_u64_kernel<<<blocks_for(L0), 256, 0, st>>>(nw.as<u64>(), first.as<u32>(), candIdx.as<u32>(), L0, cand.as<u64>());
    if (int rc = read_count(3, "finding insert branch nodes"))
      return rc;
    L = hc[3];
  }
  const u32 F = Un + L;
  TmpBuf fk, map, oldToNew, clusterNode;
  if ((e = fk.ensure(sizeof(u64) * F, st)) || (e = map.ensure(sizeof(u32) * Un, st)) || (e = oldToNew.ensure(sizeof(u32) * M, st)) ||
      (e = clusterNode.ensure(sizeof(u32) * std::max<u32>(C, 1), st)))
    return cuda_status(e, "allocating insert nodes");
  insert_place_s0_kernel<<<blocks_for(Un), 256, 0, st>>>(s0.as<u64>(), Un, cand.as<u64>(), L, fk.as<u64>(), map.as<u32>());
  if (L)
    insert_place_new_kernel<<<blocks_for(L), 256, 0, st>>>(s0.as<u64>(), Un, cand.as<u64>(), L, fk.as<u64>());
  insert_node_index_kernel<<<blocks_for(m), 256, 0, st>>>(s0Of.as<u32>(), map.as<u32>(), M, C, oldToNew.as<u32>(), clusterNode.as<u32>());
  ek.release();
  ev.release();
  idx.release();
  s0.release();
  s0Of.release();
  cand.release();
  candIdx.release();
  nw.release();
  nwVals.release();
  map.release();

  // 4. parents, child slots, link levels and breadth-first positions
  prof.mark("links", st);
  TmpBuf parent, slot, occupied, depthCount, lvlA, lvlB, ancA, ancB, order, pos, firstChild;
  if ((e = parent.ensure(sizeof(u32) * F, st)) || (e = slot.ensure(F, st)) || (e = occupied.ensure(sizeof(u32) * F, st)) ||
      (e = depthCount.ensure(sizeof(u32) * 64, st)) || (e = lvlA.ensure(sizeof(u32) * F, st)) || (e = lvlB.ensure(sizeof(u32) * F, st)) ||
      (e = ancA.ensure(sizeof(u32) * F, st)) || (e = ancB.ensure(sizeof(u32) * F, st)) || (e = order.ensure(sizeof(u32) * F, st)) ||
      (e = pos.ensure(sizeof(u32) * F, st)) || (e = firstChild.ensure(sizeof(u32) * F, st)))
    return cuda_status(e, "allocating insert links");
  cudaMemsetAsync(depthCount.p, 0, sizeof(u32) * 64, st);
  cudaMemsetAsync(occupied.p, 0, sizeof(u32) * F, st);
  insert_parents_kernel<<<blocks_for(F), 256, 0, st>>>(fk.as<u64>(), F, D, parent.as<u32>(), slot.as<unsigned char>(), occupied.as<u32>(),
                                                       depthCount.as<u32>(), err);
  insert_level_init_kernel<<<blocks_for(F), 256, 0, st>>>(parent.as<u32>(), F, lvlA.as<u32>(), ancA.as<u32>());
  for (u32 r = 0; (1u << r) <= D; ++r) // link levels are at most D
  {
    insert_level_jump_kernel<<<blocks_for(F), 256, 0, st>>>(lvlA.as<u32>(), ancA.as<u32>(), F, lvlB.as<u32>(), ancB.as<u32>());
    swap(lvlA, lvlB);
    swap(ancA, ancB);
  }
  iota_u32_kernel<<<blocks_for(F), 256, 0, st>>>(order.as<u32>(), F);
  if (int rc = sort_pairs_u32(lvlA.as<u32>(), order.as<u32>(), F, 5, st, err)) // stable: depth-first order within a level
    return rc;
  insert_positions_kernel<<<blocks_for(F), 256, 0, st>>>(order.as<u32>(), F, pos.as<u32>());
  insert_first_child_kernel<<<blocks_for(F), 256, 0, st>>>(parent.as<u32>(), slot.as<unsigned char>(), occupied.as<u32>(), pos.as<u32>(), F,
                                                           firstChild.as<u32>());
  parent.release();
  slot.release();
  lvlA.release();
  lvlB.release();
  ancA.release();
  ancB.release();
  order.release();

  // 5. entities ordered by their node (depth-first), old ones first within a node: the old entities
  // are in that order already, the new ones are sorted by node; each goes to its index plus the
  // count of the other group's entities before it
  prof.mark("entity order", st);
  TmpBuf oldOwner, newOwner, newPos, startOld, startNew;
  if ((e = oldOwner.ensure(sizeof(u32) * n, st)) || (e = newOwner.ensure(sizeof(u32) * n2, st)) || (e = newPos.ensure(sizeof(u32) * n2, st)) ||
      (e = startOld.ensure(sizeof(u32) * (u64(F) + 1), st)) || (e = startNew.ensure(sizeof(u32) * (u64(F) + 1), st)))
    return cuda_status(e, "allocating insert owners");
  insert_fill_kernel<<<blocks_for(n), 256, 0, st>>>(oldOwner.as<u32>(), n, 0u);
  insert_old_owner_kernel<<<blocks_for(M), 256, 0, st>>>(t.nodeLink.as<uint4>(), M, u32(n), oldToNew.as<u32>(), oldOwner.as<u32>());
  insert_new_owner_kernel<<<blocks_for(std::max<u32>(C, 1)), 256, 0, st>>>(clBegin.as<u32>(), clEnd.as<u32>(), C, clusterNode.as<u32>(),
                                                                          newOwner.as<u32>(), newPos.as<u32>());
  if (int rc = sort_pairs_u32(newOwner.as<u32>(), newPos.as<u32>(), n2, bit_count(F), st, err))
    return rc;
  insert_starts_kernel<<<blocks_for(n + 1), 256, 0, st>>>(oldOwner.as<u32>(), n, F, startOld.as<u32>());
  insert_starts_kernel<<<blocks_for(n2 + 1), 256, 0, st>>>(newOwner.as<u32>(), n2, F, startNew.as<u32>());

  // 6. the new tree
  prof.mark("write", st);
  DevBuf ids, geom, link, key, box, depth;
  if ((e = ids.ensure_pooled(sizeof(u32) * nt, st)) || (e = geom.ensure_pooled(sizeof(T) * 3 * nt, st)) ||
      (e = link.ensure_pooled(sizeof(uint4) * F, st)) || (e = key.ensure_pooled(sizeof(u64) * F, st)) ||
      (e = box.ensure_pooled(sizeof(T) * 6 * F, st)) || (e = depth.ensure_pooled(F, st)))
    return cuda_status(e, "allocating the inserted tree");
  insert_old_entities_kernel<T><<<blocks_for(n), 256, 0, st>>>(oldOwner.as<u32>(), u32(n), startNew.as<u32>(), t.sortedIds.as<u32>(), t.sortedGeom.as<T>(),
                                                               ids.as<u32>(), geom.as<T>());
  insert_new_entities_kernel<T><<<blocks_for(n2), 256, 0, st>>>(newOwner.as<u32>(), newPos.as<u32>(), u32(n2), startOld.as<u32>(), nv.as<u32>(), pts,
                                                                u32(n), ids.as<u32>(), geom.as<T>());
  insert_nodes_kernel<T><<<blocks_for(F), 256, 0, st>>>(pos.as<u32>(), F, fk.as<u64>(), D, startOld.as<u32>(), startNew.as<u32>(), firstChild.as<u32>(),
                                                        occupied.as<u32>(), t.nodeBox.as<T>(), t.minTab.as<T>(), t.space.as<Space<T>>(), link.as<uint4>(),
                                                        key.as<u64>(), box.as<T>(), depth.as<unsigned char>());
  prof.mark("end", st);
  std::vector<u32> dc(64);
  if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(dc.data(), depthCount.p, sizeof(u32) * 64, cudaMemcpyDeviceToHost, st)))
    return cuda_status(e, "inserting points");
  if (int rc = read_err("inserting points"))
    return rc;
  if (hostErr & kErrTimeout)
  {
    set_error("radix sort look-back wait ran out of its iteration limit");
    return OTG_ERR_TIMEOUT;
  }
  if (hostErr & kErrCapacity)
  {
    set_error("otg_tree_insert: a clustering list overflowed, or a node of the merged set lost its parent");
    return OTG_ERR_CUDA;
  }
  std::swap(t.sortedIds, ids);
  std::swap(t.sortedGeom, geom);
  std::swap(t.nodeLink, link);
  std::swap(t.nodeKey, key);
  std::swap(t.nodeBox, box);
  std::swap(t.nodeDepth, depth);
  // the replaced arrays: pooled ones freed in stream order, a Create's kept until the next Create
  for (DevBuf* b : { &ids, &geom, &link, &key, &box, &depth })
  {
    if (b->pooled)
      b->release_async(st);
    else if (b->p)
      t.retired.push_back(std::move(*b));
  }
  t.n = nt;
  t.nodeCount = F;
  t.maxNodes = F;
  t.levelCountsHost.assign(dc.begin(), dc.begin() + D + 1);
  t.sortedKeys = nullptr;
  t.inserted = true;
  t.image32 = false;
  return OTG_OK;
}

int insert_points(TreeState& t, const void* entities, u64 n2, int mem, cudaStream_t st)
{
  if (t.trees)
  {
    set_error("otg_tree_insert: not for forests");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (t.kind != OTG_KIND_POINTS)
  {
    set_error("otg_tree_insert: point trees only (box trees would also need their node geometry updated)");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (n2 == 0)
    return OTG_OK;
  if (t.n == 0)
  {
    set_error("otg_tree_insert: the tree is empty (its space is defined by a Create with entities)");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (t.n + n2 >= (u64(1) << 30))
  {
    set_error("entity count must be below 2^30");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  cudaError_t e;
  if (!t.inserted && t.sortedKeys)
  {
    // a point outside a given space has the location key 0 and sorts first; the reference keeps it
    // in a node that the root does not link
    u64 first = 0;
    if ((e = cudaMemcpyAsync(&first, t.sortedKeys, t.keys32 ? 4 : 8, cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
      return cuda_status(e, "reading the first location");
    if (first == 0)
    {
      set_error("otg_tree_insert: the tree holds points outside its space, which no node reachable from the root holds");
      return OTG_ERR_NOT_SUPPORTED;
    }
  }
  const size_t esz = t.scalar == OTG_SCALAR_F64 ? 8 : 4;
  TmpBuf hostCopy;
  const void* src = entities;
  if (mem == OTG_MEM_HOST)
  {
    if ((e = hostCopy.ensure(esz * 3 * n2, st)) || (e = cudaMemcpyAsync(hostCopy.p, entities, esz * 3 * n2, cudaMemcpyHostToDevice, st)))
      return cuda_status(e, "copying inserted points");
    src = hostCopy.p;
  }
  const bool rasterDouble = t.scalar == OTG_SCALAR_F64 || t.D >= 16;
  int rc;
  if (t.scalar == OTG_SCALAR_F64)
    rc = insert_impl<double, double>(t, static_cast<const double*>(src), n2, st);
  else if (rasterDouble)
    rc = insert_impl<float, double>(t, static_cast<const float*>(src), n2, st);
  else
    rc = insert_impl<float, float>(t, static_cast<const float*>(src), n2, st);
  if (rc == OTG_OK && (e = cudaStreamSynchronize(st)))
    return cuda_status(e, "inserting points");
  return rc;
}

} // namespace otg
