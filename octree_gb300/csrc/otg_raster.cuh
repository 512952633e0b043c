// otg_raster.cuh — exact rasterisation without per-entity FP64 arithmetic.
//
// The reference maps a coordinate x to its grid cell with FP64 (or the tree's scalar) arithmetic:
//   points (si_grid.h:145-175): pc = x - min; pc <= 0 ? 0 : min(maxRasterID, GridID(R(pc) * factor))
//   loose-box centres (si_grid.h:236-241): GridID(R(c - min) * factor)
//   loose-box levels  (si_grid.h:243-252): bit_width(ceil(max_d R(size_d) * factor_d) - 1)
// Every one of these is a monotone non-decreasing function of its input (each step is a
// round-to-nearest of a monotone operation, or a truncation). A monotone step function is
// described exactly by the smallest input at which each step is reached. These thresholds are
// found once per build by searching the ordered bit patterns of the scalar type while
// evaluating the reference formula itself; afterwards a cell is the number of thresholds at or
// below the coordinate, which takes integer compares only. GB300 executes FP64 at a small
// fraction of its FP32/integer rate, so this removes FP64 from the per-entity path while keeping
// every key bit-identical.
#pragma once

#include "otg_device.cuh"

namespace otg
{

template<typename T>
struct Ord;
template<>
struct Ord<double>
{
  using U = unsigned long long;
  static __host__ __device__ __forceinline__ U of(double v)
  {
#ifdef __CUDA_ARCH__
    U b = (U)__double_as_longlong(v);
#else
    U b;
    __builtin_memcpy(&b, &v, 8);
#endif
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
  }
  static __device__ __forceinline__ double val(U o) { return __longlong_as_double((long long)((o >> 63) ? (o & 0x7fffffffffffffffULL) : ~o)); }
  static constexpr U kNever = ~0ULL; // above the image of +inf
};
template<>
struct Ord<float>
{
  using U = unsigned int;
  static __host__ __device__ __forceinline__ U of(float v)
  {
#ifdef __CUDA_ARCH__
    U b = __float_as_uint(v);
#else
    U b;
    __builtin_memcpy(&b, &v, 4);
#endif
    return (b >> 31) ? ~b : (b | 0x80000000u);
  }
  static __device__ __forceinline__ float val(U o) { return __uint_as_float((o >> 31) ? (o & 0x7fffffffu) : ~o); }
  static constexpr U kNever = ~0u;
};

// Smallest ordered value in [image(-inf), image(+inf)] with pred true (pred monotone false -> true),
// starting the search at `guess`; Ord<T>::kNever when pred is false everywhere.
template<typename T, typename F>
__device__ typename Ord<T>::U first_true(F pred, T guess)
{
  using O = Ord<T>;
  using U = typename O::U;
  const U lo0 = O::of(-Lim<T>::max()) - 1; // image of -inf
  const U hi0 = O::of(Lim<T>::max()) + 1;  // image of +inf
  U g = O::of(guess);
  if (g < lo0)
    g = lo0;
  if (g > hi0)
    g = hi0;
  U lo, hi; // pred(lo) false, pred(hi) true
  if (pred(O::val(g)))
  {
    hi = g;
    U step = 1;
    for (;;)
    {
      if (hi - lo0 <= step)
      {
        if (pred(O::val(lo0)))
          return lo0;
        lo = lo0;
        break;
      }
      U c = hi - step;
      if (!pred(O::val(c)))
      {
        lo = c;
        break;
      }
      hi = c;
      step <<= 1;
    }
  }
  else
  {
    lo = g;
    U step = 1;
    for (;;)
    {
      if (hi0 - lo <= step)
      {
        if (!pred(O::val(hi0)))
          return O::kNever;
        hi = hi0;
        break;
      }
      U c = lo + step;
      if (pred(O::val(c)))
      {
        hi = c;
        break;
      }
      lo = c;
      step <<= 1;
    }
  }
  while (hi - lo > 1)
  {
    U mid = lo + (hi - lo) / 2;
    if (pred(O::val(mid)))
      hi = mid;
    else
      lo = mid;
  }
  return hi;
}

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

__device__ __forceinline__ u32 to_grid(double v) { return u32(v); } // C++ truncation toward zero
__device__ __forceinline__ u32 to_grid(float v) { return u32(v); }

// ---------------------------------------------------------------- reference formulas
// si_grid.h:157-170 for one dimension of a point known to be inside the space
template<typename T, typename R>
__device__ __forceinline__ u32 point_cell_ref(T x, const Space<T>& s, int d, u32 maxRasterID)
{
  T pc = x - s.min[d];
  if (pc <= 0)
    return 0;
  u32 rid = to_grid(R(pc) * Raster<R, T>::rast(s, d));
  return rid < maxRasterID ? rid : maxRasterID;
}
// si_grid.h:158: the point is outside the space (with tolerance)
template<typename T, typename R>
__device__ __forceinline__ bool point_below_ref(T x, const Space<T>& s, int d)
{
  T pc = x - s.min[d];
  return pc < -base_tol<T>();
}
template<typename T, typename R>
__device__ __forceinline__ bool point_above_ref(T x, const Space<T>& s, int d)
{
  T pc = x - s.min[d];
  return pc > Raster<R, T>::rsize(s, d) + R(base_tol<T>());
}
// si_grid.h:239-240 loose box centre cell (not clamped)
template<typename T, typename R>
__device__ __forceinline__ u32 center_cell_ref(T c, const Space<T>& s, int d)
{
  return to_grid(R(c - s.min[d]) * Raster<R, T>::rast(s, d));
}
// si_grid.h:245: relative size of one dimension
template<typename T, typename R>
__device__ __forceinline__ R rel_size_ref(T size, const Space<T>& s, int d)
{
  return R(size) * Raster<R, T>::rast(s, d);
}

// ---------------------------------------------------------------- tables
// Per dimension: [0] validity lower bound, [1] validity upper bound (inclusive), then the level
// thresholds (boxes), then the cell thresholds cell[0..cells-1] (cell[0] = 0: everything).
constexpr int kLevelThresholds = 33;

template<typename T>
struct RasterLayout
{
  using U = typename Ord<T>::U;
  u32 cells;  // thresholds per dimension (2^D for points, 2^D + 2 for box centres)
  static __host__ __device__ size_t per_dim(u32 cells) { return 2 + kLevelThresholds + cells; }
  static __host__ __device__ size_t bytes(u32 cells) { return sizeof(U) * 3 * per_dim(cells); }
};

// Threshold j of dimension d (layout above) for the space s. isBox selects the box variants.
template<typename T, typename R>
__device__ typename Ord<T>::U raster_threshold(const Space<T>& s, int d, u32 j, u32 cells, int isBox)
{
  using O = Ord<T>;
  const u32 D = s.D;
  const u32 maxRasterID = (1u << D) - 1u;
  const T dr = T(Raster<R, T>::derast(s, d));
  if (j == 0)
  {
    if (isBox) // DoesRangeContainBox lower bound: !(rmin - tol > b)  <=>  b >= rmin - tol
      return O::of(T(s.min[d] - base_tol<T>()));
    return first_true<T>([&](T x) { return !point_below_ref<T, R>(x, s, d); }, s.min[d]);
  }
  if (j == 1)
  {
    if (isBox) // !(b > rmax + tol)
      return O::of(T(s.max[d] + base_tol<T>()));
    typename O::U a = first_true<T>([&](T x) { return point_above_ref<T, R>(x, s, d); }, s.max[d]);
    return a == O::kNever ? O::of(Lim<T>::max()) + 1 : a - 1;
  }
  if (j < 2 + kLevelThresholds)
  {
    // level >= L  <=>  R(size) * factor > 2^(L - 1)
    const u32 L = j - 2;
    if (L == 0)
      return 0;
    const R lim = R(u64(1) << (L - 1));
    return first_true<T>([&](T size) { return rel_size_ref<T, R>(size, s, d) > lim; }, T(lim) * dr);
  }
  const u32 g = j - 2 - kLevelThresholds;
  if (g == 0)
    return 0;
  if (isBox)
    return first_true<T>([&](T c) { return center_cell_ref<T, R>(c, s, d) >= g; }, T(s.min[d] + T(g) * dr));
  if (g > maxRasterID)
    return O::kNever;
  return first_true<T>([&](T x) { return point_cell_ref<T, R>(x, s, d, maxRasterID) >= g; }, T(s.min[d] + T(g) * dr));
}

// One thread per (dimension, threshold index).
template<typename T, typename R>
__global__ void raster_tables_kernel(const Space<T>* __restrict__ spg, typename Ord<T>::U* __restrict__ tab, u32 cells, int isBox)
{
  const Space<T>& s = *spg;
  const size_t perDim = RasterLayout<T>::per_dim(cells);
  const u64 total = 3 * perDim;
  for (u64 idx = blockIdx.x * u64(blockDim.x) + threadIdx.x; idx < total; idx += u64(gridDim.x) * blockDim.x)
    tab[idx] = raster_threshold<T, R>(s, int(idx / perDim), u32(idx % perDim), cells, isBox);
}

// Unsigned 64-bit order with 32-bit operations only. 64-bit integer compares and selects appear to
// issue on the FP64 pipe of this GPU: in min/max reductions over every entity (bounding box) the
// 32-bit form is faster; where the compares are few and other work dominates, native compares
// overlap better.
__device__ __forceinline__ bool lt_u64(unsigned long long a, unsigned long long b)
{
  const u32 ah = u32(a >> 32), bh = u32(b >> 32);
  return ah < bh || (ah == bh && u32(a) < u32(b));
}
__device__ __forceinline__ bool lt_ord(unsigned long long a, unsigned long long b) { return lt_u64(a, b); }
__device__ __forceinline__ bool lt_ord(unsigned int a, unsigned int b) { return a < b; }

// ordered bits of a double from its two 32-bit halves (same map as Ord<double>::of)
__device__ __forceinline__ unsigned long long ord_bits(double v)
{
  const u32 hi = u32(__double2hiint(v)), lo = u32(__double2loint(v));
  const u32 s = u32(int(hi) >> 31);
  return (u64(hi ^ (s | 0x80000000u)) << 32) | u64(lo ^ s);
}
__device__ __forceinline__ unsigned int ord_bits(float v)
{
  const u32 b = __float_as_uint(v);
  return b ^ (u32(int(b) >> 31) | 0x80000000u);
}

// an FP32 value close to v (truncated from the bit pattern, no conversion instruction): estimates only
__device__ __forceinline__ float approx_f(double v)
{
  const u32 hi = u32(__double2hiint(v)), lo = u32(__double2loint(v));
  const int ex = int((hi >> 20) & 0x7ffu) - 1023 + 127;
  if (ex <= 0)
    return 0.f;
  if (ex >= 255)
    return (hi >> 31) ? -3.0e38f : 3.0e38f;
  return __uint_as_float((hi & 0x80000000u) | (u32(ex) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}
__device__ __forceinline__ float approx_f(float v) { return v; }

// number of thresholds <= o, minus one (the cell), searching around an estimate
template<typename U>
__device__ __forceinline__ u32 cell_from_table(const U* __restrict__ thr, u32 cells, U o, int estimate)
{
  u32 g = estimate < 0 ? 0u : (u32(estimate) >= cells ? cells - 1 : u32(estimate));
  if (o < thr[g])
  {
    u32 lo = 0, hi = g; // thr[lo] <= o < thr[hi]
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
  if (g + 1 < cells && o >= thr[g + 1])
  {
    u32 lo = g + 1, hi = cells; // thr[lo] <= o
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
  return g;
}

// MinPoint node table: minTab[d][(2^depth - 1) + cell] for depth 0..D (si_grid.h:124-143 and
// ot_dynamic_hash_core.h:563-572): T((R(cell << (D - depth)) + halfGrid) * derast) + min - nodeSize[depth + 1]
template<typename T, typename R>
__device__ __forceinline__ T node_min_entry(const Space<T>& s, int d, u64 j)
{
  const u32 depth = u32(63 - __clzll((long long)(j + 1)));
  const u64 cell = (j + 1) - (u64(1) << depth);
  const u32 lvl = s.D - depth;
  const R halfGrid = R(u64(1) << lvl) * R(0.5);
  const T c = T((R(u32(cell << lvl)) + halfGrid) * Raster<R, T>::derast(s, d)) + s.min[d];
  return c - s.nodeSize[depth + 1][d];
}

template<typename T, typename R>
__global__ void node_min_table_kernel(const Space<T>* __restrict__ spg, T* __restrict__ tab)
{
  const Space<T>& s = *spg;
  const u64 perDim = (u64(2) << s.D) - 1;
  for (u64 idx = blockIdx.x * u64(blockDim.x) + threadIdx.x; idx < 3 * perDim; idx += u64(gridDim.x) * blockDim.x)
    tab[idx] = node_min_entry<T, R>(s, int(idx / perDim), idx % perDim);
}

} // namespace otg
