// otg_device.cuh — device-side arithmetic shared by the build and query kernels.
//
// Every predicate here reproduces the reference's floating-point operation order exactly
// (OrthoTree, adapters/general.h and detail/internal_geometry_module.h, cited per function).
// The whole library is compiled with --fmad=false, so no a*b+c is contracted into an FMA and
// each + - * / sqrt is one IEEE round-to-nearest operation, as on the host.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace otg
{
using u32 = uint32_t;
using u64 = uint64_t;

// core/types.h:61-67
constexpr u32 kInvalidDepth = 31;

template<typename T>
struct Lim;
template<>
struct Lim<double>
{
  static __host__ __device__ constexpr double max() { return 1.7976931348623157e308; }
  static __host__ __device__ constexpr double eps() { return 2.220446049250313e-16; }
};
template<>
struct Lim<float>
{
  static __host__ __device__ constexpr float max() { return 3.402823466e38f; }
  static __host__ __device__ constexpr float eps() { return 1.192092896e-07f; }
};

// adapters/general.h:57 BASE_TOLERANCE = epsilon * 100
template<typename T>
__host__ __device__ constexpr T base_tol()
{
  return Lim<T>::eps() * T(100);
}

// std::min / std::max semantics (second argument wins only when strictly better)
template<typename T>
__host__ __device__ __forceinline__ T smin(T a, T b)
{
  return (b < a) ? b : a;
}
template<typename T>
__host__ __device__ __forceinline__ T smax(T a, T b)
{
  return (a < b) ? b : a;
}

// ------------------------------------------------------------------ Morton code
// detail/si_morton.h:450-464 Part1By2 (64-bit), 21 bits spread two apart
__host__ __device__ __forceinline__ u64 part1by2(u32 g)
{
  u64 x = g;
  x = (x ^ (x << 32)) & 0xffff00000000ffffULL;
  x = (x ^ (x << 16)) & 0x00ff0000ff0000ffULL;
  x = (x ^ (x << 8)) & 0xf00f00f00f00f00fULL;
  x = (x ^ (x << 4)) & 0x30c30c30c30c30c3ULL;
  x = (x ^ (x << 2)) & 0x9249249249249249ULL;
  return x;
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

// detail/si_morton.h:519-535 3-D Encode (x -> bit 0, y -> bit 1, z -> bit 2)
__host__ __device__ __forceinline__ u64 encode3(u32 x, u32 y, u32 z) { return (part1by2(z) << 2) + (part1by2(y) << 1) + part1by2(x); }

// The same code for grid coordinates below 2^10 (depth up to 10) in 32-bit arithmetic: the bits of
// part1by2 for 10-bit inputs, in a third of the instructions of the 64-bit spread.
__host__ __device__ __forceinline__ u32 part1by2_10(u32 g)
{
  u32 x = g & 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}
__host__ __device__ __forceinline__ u32 encode3_10(u32 x, u32 y, u32 z) { return (part1by2_10(z) << 2) | (part1by2_10(y) << 1) | part1by2_10(x); }

// detail/si_morton.h:257-263 depth of a sentinel node key
__host__ __device__ __forceinline__ u32 key_depth(u64 key)
{
#ifdef __CUDA_ARCH__
  return u32(63 - __clzll((long long)key)) / 3u;
#else
  return u32(63 - __builtin_clzll(key)) / 3u;
#endif
}

// ------------------------------------------------------------------ grid space
// Everything the build kernels need about the tree space, computed once on the device from
// the (given or reduced) box: detail/si_grid.h:65-103 and core/ot_base.h:121-134.
template<typename T>
struct Space
{
  T min[3];
  T max[3];
  T size[3];       // m_sizeInDimensions (T)
  double rsizeD[3], rastD[3], derastD[3];
  float rsizeF[3], rastF[3], derastF[3];
  T nodeSize[22][3]; // MinPoint node sizes for depth 0..D+1 (points only)
  u32 D;
  u32 rasterDouble; // float trees with D >= 16 rasterise in double (si_grid.h:70-80)
};

// ------------------------------------------------------------------ geometry predicates
template<typename T>
struct GeoD
{
  static __device__ __forceinline__ bool is_less(T a, T b, T tol) { return a + tol < b; }          // general.h:246
  static __device__ __forceinline__ bool almost_equal(T a, T b, T tol) { return fabs(a - b) <= tol; } // general.h:245

  // general.h:262-289 GetBoxRelation: -1 overlapped, 0 adjacent, 1 separated
  static __device__ __forceinline__ int box_relation(const T* e1, const T* e2, T tol)
  {
    u32 rel = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      T min1 = e1[d], max1 = e1[3 + d], min2 = e2[d], max2 = e2[3 + d];
      if (is_less(min1, max2, tol) && is_less(min2, max1, tol))
        rel |= 1u;
      else if (almost_equal(min1, max2, tol) || almost_equal(max1, min2, tol))
        rel |= 2u;
      else if (is_less(max2, min1, tol) || is_less(max1, min2, tol))
        return 1;
    }
    return (rel & 2u) ? 0 : -1;
  }
  // general.h:296-310 AreBoxesOverlapped(e1, e2, true): containment, tolerance ignored
  static __device__ __forceinline__ bool contains_box_no_tol(const T* e1, const T* e2)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      if (e1[d] > e2[d] || e2[d] > e1[3 + d])
        return false;
      if (e1[d] > e2[3 + d] || e2[3 + d] > e1[3 + d])
        return false;
    }
    return true;
  }
  // general.h:225-243 DoesBoxContainPoint
  static __device__ __forceinline__ bool box_contains_point(const T* box, const T* p, T tol)
  {
    if (tol != T(0))
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (!(box[d] - tol < p[d] && p[d] < box[3 + d] + tol))
          return false;
    }
    else
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (!(box[d] <= p[d] && p[d] <= box[3 + d]))
          return false;
    }
    return true;
  }
  // general.h:135-146 Distance2 / Distance
  static __device__ __forceinline__ T distance2(const T* a, const T* b)
  {
    T d2 = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      T v = a[d] - b[d];
      d2 += v * v;
    }
    return d2;
  }
  static __device__ __forceinline__ T distance(const T* a, const T* b) { return sqrt(distance2(a, b)); }
  // general.h:218-221
  static __device__ __forceinline__ bool points_equal(const T* a, const T* b, T tol) { return distance2(a, b) <= tol * tol; }

  // general.h:159-216 MinMaxDistance (returns min, minMax)
  static __device__ __forceinline__ void min_max_distance(const T* pt, const T* box, T tol, T& outMin, T& outMinMax)
  {
    T dmin = T(0), dminMax = T(0);
    T farthestInside2 = Lim<T>::max();
    T largestDiff = T(0);
    bool isInside = true;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      T v = pt[d], minC = box[d], maxC = box[3 + d];
      T minDist = v - minC;
      T maxDist = maxC - v;
      bool inComp = (-tol <= minDist && -tol <= maxDist);
      isInside &= inComp;
      T minDist2 = minDist * minDist;
      T maxDist2 = maxDist * maxDist;
      if (maxDist2 < minDist2)
      {
        T t = minDist2;
        minDist2 = maxDist2;
        maxDist2 = t;
      }
      if (isInside)
        farthestInside2 = smin(farthestInside2, maxDist2);
      if (!inComp)
        dmin += minDist2;
      largestDiff = smax(largestDiff, maxDist2 - minDist2);
      dminMax += maxDist2;
    }
    if (isInside)
    {
      dmin = T(0);
      dminMax = farthestInside2;
    }
    else
      dminMax -= largestDiff;
    outMin = sqrt(dmin);
    outMinMax = sqrt(dminMax);
  }

  // general.h:322-335 GetPointPlaneRelation: 0 negative, 1 hit, 2 positive
  static __device__ __forceinline__ int point_plane(const T* p, T dist, const T* n, T tol)
  {
    T proj = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      proj += n[d] * p[d];
    if (proj < dist - tol)
      return 0;
    if (proj > dist + tol)
      return 2;
    return 1;
  }
  // internal_geometry_module.h:254-280 GetBoxPlaneRelationAD (projected radius accumulates in double)
  static __device__ __forceinline__ int box_plane(const T* minPoint, const T* size, T dist, const T* n, T tol)
  {
    T center[3], half[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      half[d] = size[d] * T(0.5);
      center[d] = minPoint[d] + half[d];
    }
    double radius = double(tol);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      radius += double(half[d] * T(fabs(n[d])));
    T dot = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      dot += n[d] * center[d];
    T cproj = dot - dist;
    if constexpr (sizeof(T) == 4)
    {
      // FP32 decision with the double-accumulated radius bracketed: with tol >= 0 the four addends
      // are non-negative, so the float sum rf is within 3 * 2^-24 (plus 3 * 2^-53) of the double one.
      // rf +- rf * 2^-19 brackets it after its own rounding; only positions inside the bracket take
      // the double path below. The double instructions run on the slow FP64 pipe of this GPU.
      if (tol >= T(0))
      {
        float rf = tol;
#pragma unroll
        for (int d = 0; d < 3; ++d)
          rf += half[d] * fabsf(n[d]);
        const float e = rf * 0x1p-19f + 0x1p-126f;
        const float hi = rf + e, lo = rf - e;
        if (cproj < -hi)
          return 0;
        if (cproj > hi)
          return 2;
        if (cproj > -lo && cproj < lo)
          return 1;
      }
    }
    if (double(cproj) + radius < 0.0)
      return 0;
    if (double(cproj) - radius > 0.0)
      return 2;
    return 1;
  }
  // internal_geometry_module.h:148-161 AreBoxesOverlappingByMinPoint
  static __device__ __forceinline__ bool overlap_by_min_point(const T* minL, const T* sizeL, const T* minR, const T* sizeR, T tol)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      T maxL = minL[d] + sizeL[d];
      T maxR = minR[d] + sizeR[d];
      if (maxL <= minR[d] - tol || maxR <= minL[d] - tol)
        return false;
    }
    return true;
  }
  // internal_geometry_module.h:190-199
  static __device__ __forceinline__ bool range_contains(T rmin, T rmax, T bmin, T bmax, T tol)
  {
    if (rmin - tol > bmin || bmin > rmax + tol)
      return false;
    if (rmin - tol > bmax || bmax > rmax + tol)
      return false;
    return true;
  }
  // internal_geometry_module.h:201-237 DoesRangeContainBoxAD(range, box{min,max})
  static __device__ __forceinline__ bool range_contains_box(const T* range, const T* box, T tol)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (!range_contains(range[d], range[3 + d], box[d], box[3 + d], tol))
        return false;
    return true;
  }
  // internal_geometry_module.h:239-252 DoesRangeContainBoxAD(range, minPoint, size)
  static __device__ __forceinline__ bool range_contains_min_size(const T* range, const T* minPoint, const T* size, T tol)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      T bmax = minPoint[d] + size[d];
      if (!range_contains(range[d], range[3 + d], minPoint[d], bmax, tol))
        return false;
    }
    return true;
  }
  // internal_geometry_module.h:398-422 DoesBoxContainPointAD(minPoint, size, p): centre / half form
  static __device__ __forceinline__ bool node_contains_point(const T* minPoint, const T* size, const T* p, T tol)
  {
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      T half = size[d] * T(0.5);
      T dist = fabs(p[d] - minPoint[d] - half);
      if (tol != T(0))
      {
        if (dist >= half + tol)
          return false;
      }
      else if (dist > half)
        return false;
    }
    return true;
  }
  // internal_geometry_module.h:424-458 GetBoxWallDistanceAD(..., isInsideConsideredAsZero = true)
  static __device__ __forceinline__ T wall_distance(const T* p, const T* minPoint, const T* size)
  {
    T cd[3], half[3];
    bool inside = true;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      half[d] = size[d] * T(0.5);
      cd[d] = fabs(minPoint[d] + half[d] - p[d]);
      inside &= cd[d] <= half[d];
    }
    if (inside)
      return T(0);
    T d2 = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      T v = smax(T(0), cd[d] - half[d]);
      d2 += v * v;
    }
    return sqrt(d2);
  }
};

// ------------------------------------------------------------------ ray tester
// internal_geometry_module.h:536-723 RayHitTester
template<typename T>
struct RayD
{
  T origin[3], dir[3], inv[3];
  T minTol, tolInc;
  u32 sign;     // bit d: direction component d < 0
  u32 zero;     // bit d: |direction d| < 2 eps (treated as NaN inverse)
  bool valid;

  // internal_geometry_module.h:539-568
  __device__ void make(const T* o, const T* nd, T minTolerance, T toleranceIncrement)
  {
    T s2 = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      s2 += nd[d] * nd[d];
    valid = fabs(double(s2) - 1.0) < 0.000001; // general.h:223 IsNormalizedVector
    minTol = minTolerance;
    tolInc = toleranceIncrement;
    sign = 0;
    zero = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      origin[d] = o[d];
      dir[d] = nd[d];
      T c = nd[d];
      bool isNaN = double(fabs(c)) < 2.0 * double(Lim<T>::eps());
      inv[d] = isNaN ? T(0) : (T(1) / c);
      if (c < 0)
        sign |= 1u << d;
      if (isNaN)
        zero |= 1u << d;
    }
  }

  // internal_geometry_module.h:631-712 BoxHitTest<true>
  __device__ bool box_hit_test(const T* minDiff, const T* maxDiff, T& enterOut, T& exitOut) const
  {
    T enter = -Lim<T>::max();
    T exit = Lim<T>::max();
    if (zero)
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (!(zero & (1u << d)))
          enter = fmax(enter, ((sign >> d) & 1u) ? maxDiff[d] * inv[d] : minDiff[d] * inv[d]);
#pragma unroll
      for (int d = 0; d < 3; ++d)
        if (!(zero & (1u << d)))
          exit = fmin(exit, ((sign >> d) & 1u) ? minDiff[d] * inv[d] : maxDiff[d] * inv[d]);
    }
    else
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
        enter = smax(enter, ((sign >> d) & 1u) ? maxDiff[d] * inv[d] : minDiff[d] * inv[d]);
#pragma unroll
      for (int d = 0; d < 3; ++d)
        exit = smin(exit, ((sign >> d) & 1u) ? minDiff[d] * inv[d] : maxDiff[d] * inv[d]);
    }
    T exitTol = smax(T(0), exit) * tolInc + minTol;
    enter -= T(0.5) * (smax(T(0), enter) * tolInc + minTol);
    exit += T(0.5) * (smax(T(0), exit) * tolInc + minTol);
    if (enter >= exit || exit <= T(0))
      return false;
    enter = smax(T(0), enter);
    if (zero)
    {
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        if (!(zero & (1u << d)))
          continue;
        if (minDiff[d] > exitTol || maxDiff[d] < -exitTol)
          return false;
      }
    }
    enterOut = enter;
    exitOut = exit;
    return true;
  }
  // internal_geometry_module.h:576-585 Hit(minPoint, size)
  __device__ __forceinline__ bool hit_node(const T* minPoint, const T* size, T& en, T& ex) const
  {
    T a[3], b[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      a[d] = minPoint[d] - origin[d];
      b[d] = minPoint[d] + size[d] - origin[d];
    }
    return box_hit_test(a, b, en, ex);
  }
  // internal_geometry_module.h:587-597 Hit(box)
  __device__ __forceinline__ bool hit_box(const T* box, T& en, T& ex) const
  {
    T a[3], b[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      a[d] = box[d] - origin[d];
      b[d] = box[3 + d] - origin[d];
    }
    return box_hit_test(a, b, en, ex);
  }
  // internal_geometry_module.h:599-626 Hit(point)
  __device__ __forceinline__ bool hit_point(const T* p, T& en, T& ex) const
  {
    T v[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      v[d] = p[d] - origin[d];
    T t = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      t += v[d] * dir[d];
    T len2 = T(0);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      len2 += v[d] * v[d];
    T dist2 = smax(T(0), len2 - t * t);
    T tol = smax(T(0), t) * tolInc + minTol;
    if (dist2 <= (tol * tol) && t >= -tol)
    {
      en = smax(T(0), t - tol);
      ex = t + tol;
      return true;
    }
    return false;
  }
};

// order-preserving integer image of a double / float (for atomic min / max reductions)
__device__ __forceinline__ unsigned long long ordered_bits(double v)
{
  unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double from_ordered_bits(unsigned long long b)
{
  return __longlong_as_double((b >> 63) ? (b & 0x7fffffffffffffffULL) : ~b);
}
__device__ __forceinline__ unsigned int ordered_bits(float v)
{
  unsigned int b = __float_as_uint(v);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ordered_bits(unsigned int b) { return __uint_as_float((b >> 31) ? (b & 0x7fffffffu) : ~b); }

} // namespace otg
