// otg_oracle.hpp — CPU restatement of OrthoTree's Morton location-code tree (Create + queries).
//
// TEST INFRASTRUCTURE ONLY. This header is the checker for the GPU path: only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may build or call it.
// Nothing in octree_gb300/ includes or links it.
//
// It restates, in plain single-threaded C++, the algorithm of the reference library for the
// paths the GPU build accelerates. Every function names the reference file:line it follows
// (paths are relative to the OrthoTree project root). The restatement keeps the reference's
// arithmetic order operation by operation, so it must be compiled with -ffp-contract=off
// (aarch64 GCC contracts a*b+c into FMA by default, which changes results).
//
// Scope (3-D only, contiguous entity ids 0..N-1):
//   * OctreePoint: loose factor 1.0, MinPoint node geometry (core/configuration.h:104-105).
//   * OctreeBox:   loose factor 2.0, MBR node geometry      (core/configuration.h:107-108).
//     Non-loose box trees (loose factor 1.0, MBR) are also restated.
//   * Scalars: double (the library default) and float.
#pragma once

#include <algorithm>
#include <array>
#include <bit>
#include <cmath>
#include <cstdint>
#include <deque>
#include <functional>
#include <limits>
#include <numeric>
#include <optional>
#include <queue>
#include <unordered_map>
#include <utility>
#include <vector>
#include <thread>
#include <atomic>

namespace otg_oracle
{
using u32 = uint32_t;
using u64 = uint64_t;

// core/types.h:61-67
constexpr u32 INVALID_DEPTH = 31;
constexpr u32 INVALID_GRIDID = 0xFFFFFFFFu;

enum class RangeMode : int { Inside = 0, Overlap = 1 };          // core/types.h:83-87
enum class PlaneRel : int { Negative = 0, Hit = 1, Positive = 2 }; // core/types.h:91-96

// adapters/general.h:57  BASE_TOLERANCE = epsilon * 100
template<typename T>
constexpr T base_tolerance() { return std::numeric_limits<T>::epsilon() * T(100); }

// ---------------------------------------------------------------- Morton helpers
// detail/si_morton.h:432-471 (Part1By2, 64-bit location) — spread 21 bits two apart.
inline u64 part1by2(u32 g)
{
  u64 x = g;
  x = (x ^ (x << 32)) & 0xffff00000000ffffULL;
  x = (x ^ (x << 16)) & 0x00ff0000ff0000ffULL;
  x = (x ^ (x << 8)) & 0xf00f00f00f00f00fULL;
  x = (x ^ (x << 4)) & 0x30c30c30c30c30c3ULL;
  x = (x ^ (x << 2)) & 0x9249249249249249ULL;
  return x;
}
// detail/si_morton.h:519-535 (3-D Encode: x -> bit 0, y -> bit 1, z -> bit 2)
inline u64 encode3(const u32 g[3]) { return (part1by2(g[2]) << 2) + (part1by2(g[1]) << 1) + part1by2(g[0]); }

// detail/si_morton.h:257-263 (GetDepthID of a sentinel node key)
inline u32 key_depth(u64 key) { return u32(std::bit_width(key) - 1) / 3; }

// detail/si_morton.h:576-622 (Decode, non-BMI2 branch)
inline std::array<u32, 3> decode_node(u64 key, u32 maxDepth)
{
  std::array<u32, 3> g{ 0, 0, 0 };
  u32 depth = key_depth(key);
  u32 shift = 0;
  for (u32 lvl = maxDepth - depth; lvl < maxDepth; ++lvl)
    for (u32 d = 0; d < 3; ++d, ++shift)
      g[d] |= u32((key >> shift) & 1ULL) << lvl;
  return g;
}

// detail/si_morton.h:117-143 compact location key (loc << 5) | depth, used for D <= 19 in 3-D
inline u64 compact_key(u64 loc, u64 depth) { return (loc << 5) | depth; }
inline u32 key_loc_depth(u64 k) { return u32(k & 31u); }
inline u64 key_loc(u64 k) { return k >> 5; }

// detail/utils.h:613-622 EstimateMaxDepth (3-D, MAX_THEORETICAL_DEPTH_ID = 21)
inline u32 estimate_max_depth(size_t n, size_t maxElem)
{
  if (n <= maxElem)
    return 2;
  size_t nLeaf = n / maxElem;
  return std::clamp(static_cast<u32>(std::log2(double(nLeaf)) / 3.0), u32(2), u32(21));
}

// ---------------------------------------------------------------- geometry predicates
// All follow adapters/general.h and detail/internal_geometry_module.h line by line.
template<typename T>
struct Geo
{
  static bool is_less(T a, T b, T tol) { return a + tol < b; }                  // general.h:246
  static bool almost_equal(T a, T b, T tol) { return std::abs(a - b) <= tol; }  // general.h:245

  // general.h:262-289 GetBoxRelation: -1 overlapped, 0 adjacent, 1 separated
  static int box_relation(const T* e1, const T* e2, T tol)
  {
    unsigned rel = 0;
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
  static bool overlapped_strict(const T* e1, const T* e2, T tol) { return box_relation(e1, e2, tol) == -1; } // general.h:291-294

  // general.h:296-310 AreBoxesOverlapped(e1, e2, true, ...) — containment, tolerance ignored
  static bool contains_box_no_tol(const T* e1, const T* e2)
  {
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
  static bool box_contains_point(const T* box, const T* p, T tol)
  {
    if (tol != T(0))
    {
      for (int d = 0; d < 3; ++d)
        if (!(box[d] - tol < p[d] && p[d] < box[3 + d] + tol))
          return false;
    }
    else
    {
      for (int d = 0; d < 3; ++d)
        if (!(box[d] <= p[d] && p[d] <= box[3 + d]))
          return false;
    }
    return true;
  }

  // general.h:135-146 Distance2 / Distance
  static T distance2(const T* a, const T* b)
  {
    T d2 = T(0);
    for (int d = 0; d < 3; ++d)
    {
      T v = a[d] - b[d];
      d2 += v * v;
    }
    return d2;
  }
  static T distance(const T* a, const T* b) { return std::sqrt(distance2(a, b)); }

  // general.h:218-221 ArePointsEqual
  static bool points_equal(const T* a, const T* b, T tol) { return distance2(a, b) <= tol * tol; }

  // general.h:159-216 MinMaxDistance (box entities in kNN)
  static std::pair<T, T> min_max_distance(const T* pt, const T* box, T tol)
  {
    T dmin = T(0), dminMax = T(0);
    T farthestInside2 = std::numeric_limits<T>::max();
    T largestDiff = T(0);
    bool isInside = true;
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
        std::swap(minDist2, maxDist2);
      if (isInside)
        farthestInside2 = std::min(farthestInside2, maxDist2);
      if (!inComp)
        dmin += minDist2;
      largestDiff = std::max(largestDiff, maxDist2 - minDist2);
      dminMax += maxDist2;
    }
    if (isInside)
    {
      dmin = T(0);
      dminMax = farthestInside2;
    }
    else
      dminMax -= largestDiff;
    return { std::sqrt(dmin), std::sqrt(dminMax) };
  }

  // general.h:322-335 GetPointPlaneRelation (plane = {origoDistance, n[3]})
  static PlaneRel point_plane(const T* p, T dist, const T* n, T tol)
  {
    T proj = T{};
    for (int d = 0; d < 3; ++d)
      proj += n[d] * p[d];
    if (proj < dist - tol)
      return PlaneRel::Negative;
    if (proj > dist + tol)
      return PlaneRel::Positive;
    return PlaneRel::Hit;
  }

  // internal_geometry_module.h:254-280 GetBoxPlaneRelationAD (radius accumulates in double)
  static PlaneRel box_plane(const T* minPoint, const T* size, T dist, const T* n, T tol)
  {
    T center[3], half[3];
    for (int d = 0; d < 3; ++d)
    {
      half[d] = size[d] * T(0.5);
      center[d] = minPoint[d] + half[d];
    }
    double radius = double(tol);
    for (int d = 0; d < 3; ++d)
      radius += half[d] * std::abs(n[d]);
    T dot = T{};
    for (int d = 0; d < 3; ++d)
      dot += n[d] * center[d];
    T cproj = dot - dist;
    if (cproj + radius < 0.0)
      return PlaneRel::Negative;
    if (cproj - radius > 0.0)
      return PlaneRel::Positive;
    return PlaneRel::Hit;
  }

  // internal_geometry_module.h:148-161 AreBoxesOverlappingByMinPoint
  static bool overlap_by_min_point(const T* minL, const T* sizeL, const T* minR, const T* sizeR, T tol)
  {
    for (int d = 0; d < 3; ++d)
    {
      T maxL = minL[d] + sizeL[d];
      T maxR = minR[d] + sizeR[d];
      if (maxL <= minR[d] - tol || maxR <= minL[d] - tol)
        return false;
    }
    return true;
  }

  // internal_geometry_module.h:190-199 DoesRangeContainBox (scalar form)
  static bool range_contains(T rmin, T rmax, T bmin, T bmax, T tol)
  {
    if (rmin - tol > bmin || bmin > rmax + tol)
      return false;
    if (rmin - tol > bmax || bmax > rmax + tol)
      return false;
    return true;
  }
  // internal_geometry_module.h:201-237 DoesRangeContainBoxAD(range, box{min,max})
  static bool range_contains_box(const T* range, const T* box, T tol)
  {
    for (int d = 0; d < 3; ++d)
      if (!range_contains(range[d], range[3 + d], box[d], box[3 + d], tol))
        return false;
    return true;
  }
  // internal_geometry_module.h:239-252 DoesRangeContainBoxAD(range, minPoint, size)
  static bool range_contains_min_size(const T* range, const T* minPoint, const T* size, T tol)
  {
    for (int d = 0; d < 3; ++d)
    {
      T bmax = minPoint[d] + size[d];
      if (!range_contains(range[d], range[3 + d], minPoint[d], bmax, tol))
        return false;
    }
    return true;
  }
  // internal_geometry_module.h:372-396 DoesBoxContainPointAD(box{min,max}, p)
  static bool box_contains_point_ad(const T* box, const T* p, T tol) { return box_contains_point(box, p, tol); }
  // internal_geometry_module.h:398-422 DoesBoxContainPointAD(minPoint, size, p) (centre / half form)
  static bool node_contains_point(const T* minPoint, const T* size, const T* p, T tol)
  {
    for (int d = 0; d < 3; ++d)
    {
      T half = size[d] * T(0.5);
      T dist = std::abs(p[d] - minPoint[d] - half);
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
  // internal_geometry_module.h:424-458 GetBoxWallDistanceAD(..., isInsideConsideredAsZero=true)
  static T wall_distance(const T* p, const T* minPoint, const T* size)
  {
    T cd[3], half[3];
    bool inside = true;
    for (int d = 0; d < 3; ++d)
    {
      half[d] = size[d] * T(0.5);
      cd[d] = std::abs(minPoint[d] + half[d] - p[d]);
      inside &= cd[d] <= half[d];
    }
    if (inside)
      return T{};
    T d2 = T(0);
    for (int d = 0; d < 3; ++d)
    {
      T v = std::max(T{}, cd[d] - half[d]);
      d2 += v * v;
    }
    return std::sqrt(d2);
  }
};

// internal_geometry_module.h:536-723 RayHitTester
template<typename T>
struct RayTester
{
  T origin[3], dir[3], inv[3];
  T minTol, tolInc;
  bool sign[3], zero[3];
  bool hasNaN = false;

  // internal_geometry_module.h:539-568
  static std::optional<RayTester> make(const T* o, const T* nd, T minTolerance, T toleranceIncrement)
  {
    T s2 = T(0);
    for (int d = 0; d < 3; ++d)
      s2 += nd[d] * nd[d];
    if (!(std::abs(s2 - 1.0) < 0.000001)) // general.h:223 IsNormalizedVector
      return std::nullopt;
    RayTester r{};
    for (int d = 0; d < 3; ++d)
      r.origin[d] = o[d];
    r.minTol = minTolerance;
    r.tolInc = toleranceIncrement;
    for (int d = 0; d < 3; ++d)
      r.dir[d] = nd[d];
    for (int d = 0; d < 3; ++d)
    {
      T c = nd[d];
      bool isNaN = std::fabs(c) < 2.0 * std::numeric_limits<T>::epsilon();
      r.inv[d] = isNaN ? std::numeric_limits<T>::quiet_NaN() : (T(1) / c);
      r.sign[d] = c < 0;
      r.zero[d] = isNaN;
      r.hasNaN |= isNaN;
    }
    return r;
  }

  // internal_geometry_module.h:631-712 BoxHitTest<true>
  bool box_hit_test(const T* minDiff, const T* maxDiff, T& enterOut, T& exitOut) const
  {
    T enter = -std::numeric_limits<T>::max();
    T exit = std::numeric_limits<T>::max();
    T pd[2][3];
    for (int d = 0; d < 3; ++d)
      pd[0][d] = minDiff[d] * inv[d];
    for (int d = 0; d < 3; ++d)
      pd[1][d] = maxDiff[d] * inv[d];
    if (hasNaN)
    {
      for (int d = 0; d < 3; ++d)
        if (!zero[d])
          enter = std::fmax(enter, pd[sign[d] ? 1 : 0][d]);
      for (int d = 0; d < 3; ++d)
        if (!zero[d])
          exit = std::fmin(exit, pd[sign[d] ? 0 : 1][d]);
    }
    else
    {
      for (int d = 0; d < 3; ++d)
        enter = std::max(enter, pd[sign[d] ? 1 : 0][d]);
      for (int d = 0; d < 3; ++d)
        exit = std::min(exit, pd[sign[d] ? 0 : 1][d]);
    }
    T exitTol = std::max(T(0), exit) * tolInc + minTol;
    enter -= T(0.5) * (std::max(T(0), enter) * tolInc + minTol);
    exit += T(0.5) * (std::max(T(0), exit) * tolInc + minTol);
    if (enter >= exit || exit <= T(0))
      return false;
    enter = std::max(T(0), enter);
    if (hasNaN)
    {
      for (int d = 0; d < 3; ++d)
      {
        if (!zero[d])
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
  bool hit_node(const T* minPoint, const T* size, T& en, T& ex) const
  {
    T a[3], b[3];
    for (int d = 0; d < 3; ++d)
      a[d] = minPoint[d] - origin[d];
    for (int d = 0; d < 3; ++d)
      b[d] = minPoint[d] + size[d] - origin[d];
    return box_hit_test(a, b, en, ex);
  }
  // internal_geometry_module.h:587-597 Hit(box)
  bool hit_box(const T* box, T& en, T& ex) const
  {
    T a[3], b[3];
    for (int d = 0; d < 3; ++d)
      a[d] = box[d] - origin[d];
    for (int d = 0; d < 3; ++d)
      b[d] = box[3 + d] - origin[d];
    return box_hit_test(a, b, en, ex);
  }
  // internal_geometry_module.h:599-626 Hit(point)
  bool hit_point(const T* p, T& en, T& ex) const
  {
    T v[3];
    for (int d = 0; d < 3; ++d)
      v[d] = p[d] - origin[d];
    T t = T{};
    for (int d = 0; d < 3; ++d)
      t += v[d] * dir[d];
    T len2 = T{};
    for (int d = 0; d < 3; ++d)
      len2 += v[d] * v[d];
    T dist2 = std::max(T(0), len2 - t * t);
    T tol = std::max(T(0), t) * tolInc + minTol;
    if (dist2 <= (tol * tol) && t >= -tol)
    {
      en = std::max(T(0), t - tol);
      ex = t + tol;
      return true;
    }
    return false;
  }
};

// ---------------------------------------------------------------- the tree
template<typename T>
class Tree
{
public:
  using G = Geo<T>;
  static constexpr T TOL = base_tolerance<T>();

  struct Node
  {
    u64 key = 0;
    std::vector<u64> children; // child node keys in child-id order (ot_dynamic_hash_core.h:190-215)
    std::vector<u32> entities; // own entity ids in sorted-location order
    T minPoint[3] = { 0, 0, 0 };
    T size[3] = { 0, 0, 0 }; // MBR trees only; MinPoint trees take the per-depth table
    u64 subtreeCount = 0;
  };

  bool isBox = false;
  bool loose = false;
  u32 D = 0;
  size_t maxElem = 16;
  size_t N = 0;
  std::vector<T> geom; // N*3 (points) or N*6 (boxes: min xyz, max xyz)

  // grid space (detail/si_grid.h:65-103)
  T spaceMin[3]{}, spaceMax[3]{}, sizeT[3]{};
  bool rasterDouble = true; // float trees with D >= 16 rasterise in double (si_grid.h:70-80)
  double rsizeD[3]{}, rastD[3]{}, derastD[3]{};
  float rsizeF[3]{}, rastF[3]{}, derastF[3]{};
  u32 res = 0, maxRasterID = 0;

  std::vector<std::array<T, 3>> nodeSize; // MinPoint per-depth sizes (core/ot_base.h:121-134)
  std::unordered_map<u64, Node> nodes;
  std::vector<u64> locationKeys; // per entity, input order
  std::vector<u32> sortedOrder;  // entity ids in sorted-location order (ties by id)
  std::vector<u64> sortedKeys;   // location keys in sorted order (only while Create emits nodes)

  const T* ent(u32 id) const { return &geom[size_t(id) * (isBox ? 6 : 3)]; }

  // ------------------------------------------------------------------ space indexing
  template<typename R>
  void grid_factors(R* rsize, R* rast, R* derast)
  {
    R sub = R(res);
    for (int d = 0; d < 3; ++d)
    {
      rsize[d] = R(sizeT[d]);
      derast[d] = rsize[d] / sub;
      bool flat = rsize[d] == 0;
      rast[d] = flat ? R(1) : (sub / rsize[d]);
    }
  }

  // si_grid.h:145-175 GetPointGridID
  template<typename R>
  bool point_grid(const T* p, u32 g[3], const R* rsize, const R* rast) const
  {
    for (int d = 0; d < 3; ++d)
    {
      T pc = T(p[d]) - spaceMin[d];
      if (pc < -TOL || pc > rsize[d] + TOL)
        return false;
      if (pc <= 0)
        g[d] = 0;
      else
      {
        u32 rid = u32(R(pc) * rast[d]);
        g[d] = std::min<u32>(maxRasterID, rid);
      }
    }
    return true;
  }

  // si_grid.h:221-285 GetLooseBoxGridData<2.0>
  template<typename R>
  bool loose_box_grid(const T* box, u32 g[3], u32& level, const R* rast) const
  {
    T space[6] = { spaceMin[0], spaceMin[1], spaceMin[2], spaceMax[0], spaceMax[1], spaceMax[2] };
    if (!G::range_contains_box(space, box, TOL))
      return false;
    T center[3], bsize[3];
    for (int d = 0; d < 3; ++d)
      center[d] = (box[d] + box[3 + d]) * T(0.5); // internal_geometry_module.h:132-138
    for (int d = 0; d < 3; ++d)
      bsize[d] = T(box[3 + d] - box[d]); // internal_geometry_module.h:140-146
    for (int d = 0; d < 3; ++d)
      g[d] = u32(R(center[d] - spaceMin[d]) * rast[d]);
    R maxRel = R{};
    for (int d = 0; d < 3; ++d)
      maxRel = std::max(maxRel, R(bsize[d]) * rast[d]);
    u32 maxRelGrid = u32(std::ceil(maxRel));
    if (maxRelGrid == 0)
    {
      level = 0;
      return true;
    }
    level = u32(std::bit_width(maxRelGrid - 1));
    return true;
  }

  // si_grid.h:177-219 GetBoxGridID (non-loose trees)
  template<typename R>
  bool box_grid_range(const T* box, u32 g0[3], u32 g1[3], const R* rast) const
  {
    R zero = R{};
    R maxR = R(res);
    for (int d = 0; d < 3; ++d)
    {
      T bmin = T(box[d]) - spaceMin[d];
      T bmax = T(box[3 + d]) - spaceMin[d];
      if (bmin < -TOL || bmax > sizeT[d] + TOL)
        return false;
      R minR = R(bmin) * rast[d];
      R maxRid = R(bmax) * rast[d];
      g0[d] = u32(std::clamp(minR, zero, maxR));
      g1[d] = u32(std::clamp(maxRid, zero, maxR));
      if ((g0[d] != g1[d] && std::floor(maxRid) == maxRid) || g1[d] >= res)
        --g1[d];
    }
    return true;
  }

  // si_mortongrid.h:69-97 GetLocation -> compact key (si_morton.h:129-131)
  template<typename R>
  u64 location_key(const T* e, const R* rsize, const R* rast) const
  {
    u32 g[3];
    if (!isBox)
    {
      if (!point_grid<R>(e, g, rsize, rast))
        return compact_key(0, 0); // ALLOW_OUT_OF_SPACE_INSERTION: root (si_mortongrid.h:57-62)
      return compact_key(encode3(g), D);
    }
    if (loose)
    {
      u32 level = 0;
      if (!loose_box_grid<R>(e, g, level, rast))
        return compact_key(0, 0);
      u32 shift = level * 3;
      u64 loc = (encode3(g) >> shift) << shift;
      return compact_key(loc, u64(u32(D - level)));
    }
    u32 g1[3];
    if (!box_grid_range<R>(e, g, g1, rast))
      return compact_key(0, 0);
    // si_morton.h:698-722 GetRangeLocation
    if (g[0] == g1[0] && g[1] == g1[1] && g[2] == g1[2])
      return compact_key(encode3(g), D);
    u64 l0 = encode3(g), l1 = encode3(g1);
    u64 diff = l0 ^ l1;
    u32 levelID = (u32(std::bit_width(diff)) + 2) / 3;
    u32 shift = levelID * 3;
    return compact_key((l0 >> shift) << shift, D - levelID);
  }

  // si_grid.h:124-143 CalculateGridCellCenter, used by InitNodeGeometry (ot_dynamic_hash_core.h:563-572)
  template<typename R>
  void node_center(u64 key, T c[3], const R* derast) const
  {
    auto g = decode_node(key, D);
    u32 depth = key_depth(key);
    u32 centerLevel = D - depth;
    R halfGrid = R(u64(1) << centerLevel) * R(0.5);
    for (int d = 0; d < 3; ++d)
      c[d] = T((R(g[d]) + halfGrid) * derast[d]) + spaceMin[d];
  }

  void init_min_point(Node& n) const
  {
    T c[3];
    if (rasterDouble)
      node_center<double>(n.key, c, derastD);
    else
      node_center<float>(n.key, c, derastF);
    u32 depth = key_depth(n.key);
    for (int d = 0; d < 3; ++d)
      n.minPoint[d] = c[d] - nodeSize[depth + 1][d];
  }

  // ------------------------------------------------------------------ Create
  // ot_dynamic_hash_core.h:751-809
  void create(const T* entities, size_t n, u32 maxDepthIn, const T* box, size_t maxElemIn, bool isBoxTree, bool looseTree)
  {
    isBox = isBoxTree;
    loose = isBoxTree && looseTree;
    N = n;
    maxElem = maxElemIn;
    geom.assign(entities, entities + n * (isBox ? 6 : 3));
    nodes.clear();
    locationKeys.clear();
    sortedOrder.clear();

    // :759 box space: given, else IGM::GetBoundingBoxAD (internal_geometry_module.h:342-370)
    if (box)
    {
      for (int d = 0; d < 3; ++d)
      {
        spaceMin[d] = box[d];
        spaceMax[d] = box[3 + d];
      }
    }
    else
    {
      for (int d = 0; d < 3; ++d)
      {
        spaceMin[d] = std::numeric_limits<T>::max();
        spaceMax[d] = -std::numeric_limits<T>::max();
      }
      for (size_t i = 0; i < n; ++i)
      {
        const T* e = ent(u32(i));
        for (int d = 0; d < 3; ++d)
        {
          spaceMin[d] = std::min(spaceMin[d], e[d]);
          spaceMax[d] = std::max(spaceMax[d], isBox ? e[3 + d] : e[d]);
        }
      }
    }
    // :762-764
    D = (maxDepthIn == 0) ? estimate_max_depth(n, maxElem) : maxDepthIn;

    // InitBase :611-626 -> si_grid.h:65-103, ot_base.h:102-134
    res = u32(1) << D;
    maxRasterID = res - 1;
    for (int d = 0; d < 3; ++d)
      sizeT[d] = spaceMax[d] - spaceMin[d];
    rasterDouble = !(std::is_same_v<T, float> && D < 16);
    grid_factors<double>(rsizeD, rastD, derastD);
    grid_factors<float>(rsizeF, rastF, derastF);
    if (!isBox)
    {
      nodeSize.assign(D + 2, {});
      T lf = T(1.0);
      for (u32 d = 0; d < D + 2; ++d, lf *= T(0.5))
        for (int c = 0; c < 3; ++c)
          nodeSize[d][c] = sizeT[c] * lf;
    }
    Node root;
    root.key = 1;
    if (!isBox)
      init_min_point(root);
    else
    {
      // ot_dynamic_hash_core.h:573-576 MBR init: minPoint = {max, 0, 0}, size = 0
      root.minPoint[0] = std::numeric_limits<T>::max();
    }
    if (n == 0)
    {
      nodes.emplace(1, root);
      return;
    }

    // :774-783 locations (std::transform with the execution policy: `threads` workers)
    locationKeys.resize(n);
    parallel_ranges(n, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i)
        locationKeys[i] = rasterDouble ? location_key<double>(ent(u32(i)), rsizeD, rastD) : location_key<float>(ent(u32(i)), rsizeF, rastF);
    });

    // :791-796 sort by location (ParExec path): contiguous (location, id) records, as the
    // reference sorts its zip of Location and EntityID. Ties are ordered by id here; the
    // reference's std::sort leaves them unspecified, so every comparison is made on canonical
    // (sorted) id sets. With several workers: sorted chunks merged pairwise, each round's merges
    // in parallel.
    std::vector<std::pair<u64, u32>> kv(n);
    parallel_ranges(n, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i)
        kv[i] = { locationKeys[i], u32(i) };
    });
    const size_t chunks = std::min<size_t>(threads, std::max<size_t>(1, n / 4096));
    std::vector<size_t> cut(chunks + 1);
    for (size_t c = 0; c <= chunks; ++c)
      cut[c] = n * c / chunks;
    run_workers(chunks, [&](size_t c) { std::sort(kv.begin() + cut[c], kv.begin() + cut[c + 1]); });
    std::vector<std::pair<u64, u32>> tmp(chunks > 1 ? n : 0);
    for (size_t width = 1; width < chunks; width *= 2)
    {
      run_workers((chunks + 2 * width - 1) / (2 * width), [&](size_t m) {
        const size_t lo = cut[2 * width * m], mid = cut[std::min(chunks, 2 * width * m + width)], hi = cut[std::min(chunks, 2 * width * (m + 1))];
        std::merge(kv.begin() + lo, kv.begin() + mid, kv.begin() + mid, kv.begin() + hi, tmp.begin() + lo);
        std::copy(tmp.begin() + lo, tmp.begin() + hi, kv.begin() + lo);
      });
    }
    std::vector<u32> order(n);
    sortedKeys.resize(n);
    parallel_ranges(n, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i)
      {
        sortedKeys[i] = kv[i].first;
        order[i] = kv[i].second;
      }
    });
    std::vector<std::pair<u64, u32>>().swap(kv);

    // :800 the node map is reserved for EstimateNodeNumber nodes; :717-747 BuildSubtree
    // (depth-first emission) over the sorted records
    nodes.reserve(estimate_node_number(n, D, maxElem));
    build_subtree(std::move(root), 0, order, 0, n);
    sortedOrder = std::move(order);
    std::vector<u64>().swap(sortedKeys);

    // :803-806 node geometry
    if (isBox)
      init_mbr(nodes.at(1));
    else if (box)
      init_root_box_min_point();
  }

  // Workers for the steps the reference runs with its execution policy (location transform, sort);
  // 1 = the sequential path. BuildSubtree stays sequential, as in the reference.
  unsigned threads = 1;
  template<typename F>
  void run_workers(size_t count, F&& f) const
  {
    if (count <= 1 || threads <= 1)
    {
      for (size_t i = 0; i < count; ++i)
        f(i);
      return;
    }
    std::vector<std::thread> pool;
    std::atomic<size_t> next{ 0 };
    for (unsigned w = 0; w < std::min<size_t>(threads, count); ++w)
      pool.emplace_back([&] {
        for (size_t i; (i = next.fetch_add(1)) < count;)
          f(i);
      });
    for (auto& t : pool)
      t.join();
  }
  template<typename F>
  void parallel_ranges(size_t n, F&& f) const
  {
    const size_t parts = std::min<size_t>(threads, std::max<size_t>(1, n / 4096));
    run_workers(parts, [&](size_t p) { f(n * p / parts, n * (p + 1) / parts); });
  }

  // detail/utils.h:587-611 EstimateNodeNumber (3-D): the node map's reserved size in Create
  static size_t estimate_node_number(size_t elementNo, u32 maxDepthID, size_t maxElementNo)
  {
    if (elementNo < 10)
      return 10;
    if ((maxDepthID + 1) * 3 < 64)
    {
      const size_t nMaxChild = size_t(1) << (maxDepthID * 3);
      if (elementNo / nMaxChild > maxElementNo / 2)
        return nMaxChild;
    }
    const float nElementInNodeAvg = float(elementNo) / float(maxElementNo);
    const u32 nDepthEstimated = std::min(maxDepthID, u32(std::ceil((std::log2(nElementInNodeAvg) + 1.0) / 3.0f)));
    if (nDepthEstimated * 3 < 64)
      return size_t(1.05 * double(u64(1) << (nDepthEstimated * 3)));
    return size_t(1.5 * nElementInNodeAvg);
  }

  // ot_dynamic_hash_core.h:647-747 (ProcessNode / CreateProcessingData / BuildSubtree)
  void build_subtree(Node node, u32 depth, const std::vector<u32>& order, size_t b, size_t e)
  {
    size_t count = e - b;
    node.subtreeCount = count;
    size_t it = b;
    if (count > 0)
    {
      size_t stuckEnd = e;
      if (count > maxElem && depth < D)
      {
        // :660-666 partition_point on "entity depth == node depth" (stuck entities come first)
        stuckEnd = b;
        while (stuckEnd < e && key_loc_depth(sortedKeys[stuckEnd]) == depth)
          ++stuckEnd;
      }
      for (size_t i = b; i < stuckEnd; ++i)
        node.entities.push_back(order[i]);
      it = stuckEnd;
      while (it < e)
      {
        // :695-714 child id from bits [3(D-d-1), 3(D-d-1)+3)
        u32 examined = D - (depth + 1);
        u64 loc = key_loc(sortedKeys[it]);
        u64 mask = u64(7) << (examined * 3);
        u64 flag = loc & mask;
        u64 childID = flag >> (examined * 3);
        size_t end = it;
        while (end < e && (key_loc(sortedKeys[end]) & mask) == flag)
          ++end;
        Node child;
        child.key = (node.key << 3) | childID;
        if (!isBox)
          init_min_point(child);
        // LinkChild (ot_dynamic_hash_core.h:190-215) overwrites an existing link with the same
        // child id. That only happens when an entity's location lies outside the 3*D-bit grid (a
        // degenerate loose box centred on the max face rasterises to 2^D): the reference then
        // builds a second instance of the child whose final emplace fails, so the entity ends up
        // in nodes that are not reachable from the root. The restatement does the same.
        if (std::find(node.children.begin(), node.children.end(), child.key) == node.children.end())
          node.children.push_back(child.key);
        build_subtree(std::move(child), depth + 1, order, it, end);
        it = end;
      }
    }
    nodes.emplace(node.key, std::move(node));
  }

  // ot_dynamic_hash_core.h:1425-1450 InitializeSubtreeMinimalNodeGeometry
  void init_mbr(Node& node, T outMin[3] = nullptr, T outMax[3] = nullptr)
  {
    T bmin[3], bmax[3];
    for (int d = 0; d < 3; ++d)
    {
      bmin[d] = std::numeric_limits<T>::max();
      bmax[d] = -std::numeric_limits<T>::max();
    }
    for (u64 ck : node.children)
    {
      T cmin[3], cmax[3];
      init_mbr(nodes.at(ck), cmin, cmax);
      for (int d = 0; d < 3; ++d)
      {
        bmin[d] = std::min(bmin[d], cmin[d]);
        bmax[d] = std::max(bmax[d], cmax[d]);
      }
    }
    for (u32 id : node.entities)
    {
      const T* e = ent(id);
      for (int d = 0; d < 3; ++d)
      {
        bmin[d] = std::min(bmin[d], e[d]);
        bmax[d] = std::max(bmax[d], e[3 + d]);
      }
    }
    for (int d = 0; d < 3; ++d)
    {
      node.minPoint[d] = bmin[d];
      node.size[d] = bmax[d] - bmin[d];
    }
    if (outMin)
      for (int d = 0; d < 3; ++d)
      {
        outMin[d] = bmin[d];
        outMax[d] = bmax[d];
      }
  }

  // ot_dynamic_hash_core.h:1573-1601 InitializeRootNodeBox (MinPoint, out-of-space allowed)
  void init_root_box_min_point()
  {
    Node& root = nodes.at(1);
    T bmin[3], bmax[3];
    for (int d = 0; d < 3; ++d)
    {
      bmin[d] = root.minPoint[d];
      bmax[d] = root.minPoint[d] + nodeSize[0][d];
    }
    for (u32 id : root.entities)
    {
      const T* p = ent(id);
      for (int d = 0; d < 3; ++d)
      {
        bmin[d] = std::min(bmin[d], p[d]);
        bmax[d] = std::max(bmax[d], p[d]);
      }
    }
    for (int d = 0; d < 3; ++d)
    {
      root.minPoint[d] = bmin[d];
      nodeSize[0][d] = bmax[d] - bmin[d];
    }
  }

  // ------------------------------------------------------------------ static linear layout
  // StaticLinearOrthoTreeCore (core/ot_static_linear_core.h) over the same sorted locations: the
  // parallel Create (:524-600: locations sorted, so every child group is one run), Build (:419-521:
  // breadth first; a node with more than maxElem entities below max depth keeps its entities of
  // its own depth and splits the rest by the digit of the next level; each group becomes a node at
  // the lowest common ancestor of its locations, detail/si_morton.h:347-387), CreateNode
  // (:383-414: child segment begins only up to the last node with children) and the node geometry
  // (:346-366 MinPoint; :281-325 MBR, a node's entities and then its children's min + size).
  struct StaticLayout
  {
    std::vector<u32> childBegins;         // nodeChildSegmentBegins as stored
    std::vector<u32> segBegin, segLength; // nodeEntitySegment
    std::vector<unsigned char> depth;     // m_nodeDepthIDs
    std::vector<u32> entityStorage;       // m_entityStorage
    std::vector<T> geometry;              // per node: MinPoint (3) or MBR min and size (6)
  };

  // False where the layout is undefined: a point tree holding points outside its space. Their
  // location is the root's (depth 0, si_mortongrid.h:57-62), they lead the group of child 0, and a
  // group placed at its first location's depth would be placed at depth 0 again and again.
  bool static_layout(StaticLayout& s) const
  {
    s = StaticLayout{};
    if (N == 0)
      return true; // :539-540: no node at all
    if (!isBox)
      for (size_t i = 0; i < N; ++i)
        if (key_loc_depth(locationKeys[i]) != D)
          return false;
    auto keyAt = [&](size_t pos) { return locationKeys[sortedOrder[pos]]; };
    struct Item
    {
      u64 loc;
      u32 depth;
      u32 begin, count;
    };
    std::deque<Item> queue;
    queue.push_back({ 0, 0, 0, u32(N) });
    s.childBegins.push_back(1);
    auto createNode = [&](const Item& it, u32 ownCount, u32 childCount) {
      const u32 id = u32(s.depth.size());
      s.depth.push_back((unsigned char)it.depth);
      s.segBegin.push_back(it.begin);
      s.segLength.push_back(ownCount);
      if (childCount > 0)
      {
        s.childBegins.resize(id + 2, s.childBegins.back());
        s.childBegins.back() += childCount;
      }
      if (!isBox)
      {
        Node tmp;
        tmp.key = (u64(1) << (3 * it.depth)) | (it.loc >> (3 * (D - it.depth)));
        init_min_point(tmp);
        s.geometry.insert(s.geometry.end(), tmp.minPoint, tmp.minPoint + 3);
      }
    };
    while (!queue.empty())
    {
      const Item it = queue.front();
      queue.pop_front();
      if (it.count <= maxElem || it.depth >= D)
      {
        createNode(it, it.count, 0);
        continue;
      }
      u32 pos = it.begin;
      const u32 end = it.begin + it.count;
      u32 stuck = 0;
      if (isBox)
      {
        while (pos < end && key_loc_depth(keyAt(pos)) == it.depth)
          ++pos;
        stuck = pos - it.begin;
        if (stuck == it.count)
        {
          createNode(it, it.count, 0);
          continue;
        }
      }
      const u32 examined = D - (it.depth + 1);
      const u64 mask = u64(7) << (3 * examined);
      u32 children = 0;
      while (pos < end)
      {
        const u64 pivot = keyAt(pos);
        const u64 flag = key_loc(pivot) & mask;
        u32 minDepth = key_loc_depth(pivot);
        u64 diff = 0;
        u32 e = pos;
        while (e < end && (key_loc(keyAt(e)) & mask) == flag)
        {
          if (isBox)
            minDepth = std::min(minDepth, key_loc_depth(keyAt(e)));
          diff |= key_loc(pivot) ^ key_loc(keyAt(e));
          ++e;
        }
        const u32 levelDiff = (u32(std::bit_width(diff)) + 2) / 3;
        queue.push_back({ key_loc(pivot), std::min(minDepth, D - levelDiff), pos, e - pos });
        ++children;
        pos = e;
      }
      createNode(it, stuck, children);
    }
    s.entityStorage = sortedOrder;
    if (isBox)
    {
      // children have larger ids than their parent, so one pass from the last node up suffices
      const size_t M = s.depth.size();
      s.geometry.assign(M * 6, T(0));
      for (size_t id = M; id-- > 0;)
      {
        T bmin[3], bmax[3];
        for (int d = 0; d < 3; ++d)
        {
          bmin[d] = std::numeric_limits<T>::max();
          bmax[d] = -std::numeric_limits<T>::max();
        }
        for (u32 j = s.segBegin[id]; j < s.segBegin[id] + s.segLength[id]; ++j)
        {
          const T* e = ent(s.entityStorage[j]);
          for (int d = 0; d < 3; ++d)
          {
            bmin[d] = std::min(bmin[d], e[d]);
            bmax[d] = std::max(bmax[d], e[3 + d]);
          }
        }
        if (id + 1 < s.childBegins.size())
          for (u32 c = s.childBegins[id]; c < s.childBegins[id + 1]; ++c)
          {
            const T* g = &s.geometry[size_t(c) * 6];
            for (int d = 0; d < 3; ++d)
            {
              bmin[d] = std::min(bmin[d], g[d]);
              bmax[d] = std::max(bmax[d], T(g[d] + g[3 + d]));
            }
          }
        for (int d = 0; d < 3; ++d)
        {
          s.geometry[id * 6 + d] = bmin[d];
          s.geometry[id * 6 + 3 + d] = bmax[d] - bmin[d];
        }
      }
    }
    return true;
  }

  // ------------------------------------------------------------------ bulk Insert (point trees)
  // ot_dynamic_hash_core.h:1012-1333 Insert(newEntities, existingEntities) for OctreePoint (location
  // depth is not element specific: LowestCommonAncestorCalculator<false>, no stuck entities), then
  // LinkOrphanNodes (:826-863); MinPoint trees need no geometry update (UpdateNodeGeometry, :866-1005,
  // only unites MBRs). New entity i gets id N + i.
  // The reference partitions its buffer in place (MSD radix partition, 9-bit digits, :1102-1199) and
  // sorts ranges of at most 256 (:1310-1320). Every bucket is a run of the buffer sorted by location,
  // and a bucket's fold (the lowest common ancestor of its locations, :1153-1191) and a walk's
  // clusters depend only on the locations of the run, so this restatement sorts the buffer once
  // (ties by id) and runs the same work stack (LIFO, buckets pushed in ascending digit order) over it.
  // Returns false without inserting anything when a new point lies outside the tree's space (the
  // reference would give it the root's location with a code of 0).
  static u64 node_lca(u64 a, u64 b) // si_morton.h:307-325
  {
    if (a == b)
      return a;
    const u32 da = key_depth(a), db = key_depth(b);
    if (da > db)
      a >>= 3 * (da - db);
    else if (db > da)
      b >>= 3 * (db - da);
    const u32 levels = u32((std::bit_width(a ^ b) + 2) / 3);
    return a >> (3 * levels);
  }
  static u32 nondirect_child_id(u64 parent, u64 child) // si_morton.h:651-658
  {
    return u32((child >> (3 * (key_depth(child) - key_depth(parent) - 1))) & 7u);
  }
  // LinkChild with a non-direct child: the child of `slot` becomes `child` (children kept in slot order)
  void link_child(Node& p, u64 child)
  {
    const u32 slot = nondirect_child_id(p.key, child);
    for (auto& c : p.children)
      if (nondirect_child_id(p.key, c) == slot)
      {
        c = child;
        return;
      }
    p.children.push_back(child);
    std::sort(p.children.begin(), p.children.end(), [&](u64 a, u64 b) { return nondirect_child_id(p.key, a) < nondirect_child_id(p.key, b); });
  }
  u64 child_in_slot(const Node& p, u32 slot) const
  {
    for (u64 c : p.children)
      if (nondirect_child_id(p.key, c) == slot)
        return c;
    return 0;
  }

  bool insert_points(const T* ent, size_t n2)
  {
    if (isBox)
      return false;
    if (n2 == 0)
      return true;
    std::vector<u64> keys(n2);
    for (size_t i = 0; i < n2; ++i)
    {
      keys[i] = rasterDouble ? location_key<double>(ent + 3 * i, rsizeD, rastD) : location_key<float>(ent + 3 * i, rsizeF, rastF);
      if (key_loc_depth(keys[i]) != D)
        return false;
    }
    std::vector<std::pair<u64, u32>> buf(n2); // (location code, entity id)
    for (size_t i = 0; i < n2; ++i)
      buf[i] = { key_loc(keys[i]), u32(N + i) };
    geom.insert(geom.end(), ent, ent + 3 * n2);
    locationKeys.insert(locationKeys.end(), keys.begin(), keys.end());
    N += n2;
    std::sort(buf.begin(), buf.end());

    constexpr u32 kRadixBits = 9, kSortThreshold = 256; // :1097-1099, :1028
    auto fold_depth = [&](u64 diff) { return std::min(D, D - u32((std::bit_width(diff) + 2) / 3)); };
    std::vector<u64> orphans;
    // emitCluster (:1203-1234): the entities join the node of the location, created if missing
    auto emit = [&](size_t b, size_t e, u64 loc, u32 depth) {
      if (e == b)
        return;
      const u64 key = (u64(1) << (3 * depth)) | (loc >> (3 * (D - depth)));
      auto [it, inserted] = nodes.try_emplace(key);
      if (inserted)
      {
        it->second.key = key;
        init_min_point(it->second);
        orphans.push_back(key);
      }
      for (size_t i = b; i < e; ++i)
        it->second.entities.push_back(buf[i].second);
    };
    // emitSortedRange (:1237-1291): greedy clusters over a sorted run
    auto walk = [&](size_t b, size_t e) {
      size_t cb = b;
      while (cb < e)
      {
        const u64 base = buf[cb].first;
        u64 diff = 0;
        size_t ce = cb + 1;
        while (ce < e)
        {
          const u64 nd = diff | (base ^ buf[ce].first);
          const u32 newDepth = fold_depth(nd);
          if (ce - cb + 1 > maxElem && newDepth < D && newDepth < fold_depth(diff))
            break;
          diff = nd;
          ++ce;
        }
        emit(cb, ce, base, fold_depth(diff));
        cb = ce;
      }
    };
    struct Work
    {
      size_t b, e;
      u32 bits;
      u64 loc;
      u32 depth;
    };
    std::vector<Work> stack{ { 0, n2, 3 * D, 0, 0 } }; // the root location (:1295)
    while (!stack.empty())
    {
      const Work w = stack.back();
      stack.pop_back();
      const size_t num = w.e - w.b;
      if (num == 0)
        continue;
      if (num <= maxElem) // :1304-1308
      {
        emit(w.b, w.e, w.loc, w.depth);
        continue;
      }
      if (num <= kSortThreshold || w.bits == 0) // :1310-1317
      {
        walk(w.b, w.e);
        continue;
      }
      // radixPartition (:1153-1199): buckets of the next min(9, bits) bits, each with its fold
      const u32 numBits = std::min(kRadixBits, w.bits);
      const u32 shift = w.bits - numBits;
      const u64 mask = (u64(1) << numBits) - 1;
      size_t bb = w.b;
      while (bb < w.e)
      {
        const u64 dig = (buf[bb].first >> shift) & mask;
        size_t be = bb + 1;
        u64 diff = 0;
        while (be < w.e && ((buf[be].first >> shift) & mask) == dig)
        {
          diff |= buf[bb].first ^ buf[be].first;
          ++be;
        }
        const u32 depth = fold_depth(diff);
        stack.push_back({ bb, be, std::min((D - depth) * 3, shift), buf[bb].first, depth });
        bb = be;
      }
    }

    // LinkOrphanNodes (:826-863)
    for (size_t i = 0; i < orphans.size(); ++i)
    {
      const u64 o = orphans[i];
      u64 pk = o >> 3; // GetParentIt (:1379-1390): the nearest ancestor in the node map
      while (pk > 1 && !nodes.count(pk))
        pk >>= 3;
      Node& parent = nodes.at(pk);
      const u64 c = child_in_slot(parent, nondirect_child_id(pk, o));
      if (!c)
      {
        link_child(parent, o);
        continue;
      }
      const u64 lca = node_lca(c, o);
      if (lca == o)
      {
        link_child(parent, o);
        Node& on = nodes.at(o);
        const u64 prev = child_in_slot(on, nondirect_child_id(o, c));
        if (prev)
          orphans.push_back(prev);
        link_child(on, c);
      }
      else
      {
        link_child(parent, lca);
        auto [it, inserted] = nodes.try_emplace(lca);
        if (inserted)
        {
          it->second.key = lca;
          init_min_point(it->second);
        }
        link_child(it->second, c);
        link_child(it->second, o);
      }
    }
    return true;
  }

  // ------------------------------------------------------------------ query work counters
  // The work of the reference's traversal, counted while `countWork` is set (single-threaded use):
  // node records read (node tests), entity records read (entity tests) and ids returned. They give
  // the algorithmic bytes of a query batch: nodes x node record + entities x entity record + ids x 4.
  struct QueryWork
  {
    u64 nodes = 0, entities = 0, ids = 0;
  };
  mutable QueryWork work;
  bool countWork = false;

  // ------------------------------------------------------------------ node accessors
  // ot_dynamic_hash_core.h:491-529
  const T* node_min(const Node& n) const { return n.minPoint; }
  const T* node_size(const Node& n) const { return isBox ? n.size : nodeSize[key_depth(n.key)].data(); }
  void node_box(const Node& n, T box[6]) const
  {
    const T* mn = node_min(n);
    const T* sz = node_size(n);
    for (int d = 0; d < 3; ++d)
    {
      box[d] = mn[d];
      box[3 + d] = mn[d] + sz[d];
    }
  }
  const Node& root() const { return nodes.at(1); }

  template<typename F>
  void dfs(F&& visit, const Node& start) const
  {
    std::vector<const Node*> stack{ &start };
    while (!stack.empty())
    {
      const Node* n = stack.back();
      stack.pop_back();
      if (!visit(*n))
        continue;
      for (u64 ck : n->children)
        stack.push_back(&nodes.at(ck));
    }
  }
  void collect_subtree(const Node& n, std::vector<u32>& out) const
  {
    dfs(
      [&](const Node& m) {
        out.insert(out.end(), m.entities.begin(), m.entities.end());
        return true;
      },
      n);
  }

  // ------------------------------------------------------------------ queries
  // ot_query.h:476-583 RangeSearch
  std::vector<u32> range_search(const T* range, RangeMode mode, T tol) const
  {
    std::vector<u32> found;
    T rootBox[6];
    node_box(root(), rootBox);
    if (G::range_contains_box(range, rootBox, tol))
    {
      found.resize(N);
      std::iota(found.begin(), found.end(), 0u);
      return found;
    }
    T vol = T(1.0);
    for (int d = 0; d < 3; ++d)
      vol *= T(range[3 + d] - range[d]);
    if (vol <= 0.0)
      return found;
    T rmin[3], rsize[3];
    for (int d = 0; d < 3; ++d)
    {
      rmin[d] = range[d];
      rsize[d] = T(range[3 + d] - range[d]);
    }
    dfs(
      [&](const Node& n) {
        const T* mn = node_min(n);
        const T* sz = node_size(n);
        if (countWork)
          ++work.nodes;
        if (!G::overlap_by_min_point(rmin, rsize, mn, sz, tol))
          return false;
        if (G::range_contains_min_size(range, mn, sz, tol))
        {
          collect_subtree(n, found);
          return false;
        }
        if (countWork)
          work.entities += n.entities.size();
        for (u32 id : n.entities)
        {
          const T* e = ent(id);
          bool ok;
          if (!isBox)
            ok = G::box_contains_point(range, e, tol);
          else if (mode == RangeMode::Overlap)
            ok = G::overlapped_strict(range, e, tol);
          else
            ok = G::contains_box_no_tol(range, e);
          if (ok)
            found.push_back(id);
        }
        return true;
      },
      root());
    if (countWork)
      work.ids += found.size();
    return found;
  }

  // ot_query.h:425-466 PickSearch
  std::vector<u32> pick_search(const T* p, T tol) const
  {
    std::vector<u32> found;
    T rootBox[6];
    node_box(root(), rootBox);
    if (!G::box_contains_point_ad(rootBox, p, tol))
      return found;
    dfs(
      [&](const Node& n) {
        if (!G::node_contains_point(node_min(n), node_size(n), p, tol))
          return false;
        for (u32 id : n.entities)
        {
          bool ok = isBox ? G::box_contains_point(ent(id), p, tol) : G::points_equal(ent(id), p, tol);
          if (ok)
            found.push_back(id);
        }
        return true;
      },
      root());
    if (countWork)
      work.ids += found.size();
    return found;
  }

  // relation of one entity to a plane: ot_query.h:586-602 GetEntityPlaneRelation
  PlaneRel entity_plane(u32 id, const T* pl, T tol) const
  {
    if (isBox)
    {
      const T* b = ent(id);
      T bsize[3] = { T(b[3] - b[0]), T(b[4] - b[1]), T(b[5] - b[2]) };
      return G::box_plane(b, bsize, pl[0], pl + 1, tol);
    }
    return G::point_plane(ent(id), pl[0], pl + 1, tol);
  }

  // ot_query.h:612-636 PlaneSearch (plane: {origoDistance, nx, ny, nz}): nodes the plane hits, their
  // entities the plane hits
  std::vector<u32> plane_search(const T* pl, T tol) const
  {
    std::vector<u32> found;
    dfs(
      [&](const Node& n) {
        if (G::box_plane(node_min(n), node_size(n), pl[0], pl + 1, tol) != PlaneRel::Hit)
          return false;
        for (u32 id : n.entities)
          if (entity_plane(id, pl, tol) == PlaneRel::Hit)
            found.push_back(id);
        return true;
      },
      root());
    return found;
  }

  // ot_query.h:687-744 PlanePositiveSegmentation: a node on the positive side gives its whole subtree
  // untested, a node the plane hits gives its entities that are not on the negative side
  std::vector<u32> plane_positive(const T* pl, T tol) const
  {
    std::vector<u32> found;
    dfs(
      [&](const Node& n) {
        const PlaneRel r = G::box_plane(node_min(n), node_size(n), pl[0], pl + 1, tol);
        if (r == PlaneRel::Negative)
          return false;
        if (r == PlaneRel::Positive)
        {
          collect_subtree(n, found);
          return false;
        }
        for (u32 id : n.entities)
          if (entity_plane(id, pl, tol) != PlaneRel::Negative)
            found.push_back(id);
        return true;
      },
      root());
    return found;
  }

  // one condition of Query (ot_query.h:835-861): kind 0 frustum (planes [first, first + count),
  // each with its crossing flag), 1 range Inside, 2 range Overlap (box `first`), 3 plane intersection
  // (plane `first`, own tolerance tol, < 0: the default)
  struct Cond
  {
    int kind;
    u32 first;
    u32 count;
    double tol;
  };
  static constexpr int kCondFrustum = 0, kCondRangeInside = 1, kCondRangeOverlap = 2, kCondPlane = 3;

  // ot_query.h:893-916 node selection of one condition
  bool cond_node(const Cond& c, const Node& n, const T* planes, const T* boxes, T tol) const
  {
    if (c.kind == kCondFrustum)
    {
      for (u32 i = c.first; i < c.first + c.count; ++i)
      {
        const PlaneRel r = G::box_plane(node_min(n), node_size(n), planes[4 * i], planes + 4 * i + 1, tol);
        if (r == PlaneRel::Hit)
          return true;
        if (r == PlaneRel::Negative)
          return false;
      }
      return true;
    }
    if (c.kind == kCondPlane)
    {
      const T ptol = c.tol < 0 ? base_tolerance<T>() : T(c.tol);
      return G::box_plane(node_min(n), node_size(n), planes[4 * c.first], planes + 4 * c.first + 1, ptol) == PlaneRel::Hit;
    }
    const T* r = boxes + 6 * u64(c.first);
    T rsize[3] = { T(r[3] - r[0]), T(r[4] - r[1]), T(r[5] - r[2]) };
    return G::overlap_by_min_point(r, rsize, node_min(n), node_size(n), tol);
  }

  // ot_query.h:949-998 entity selection of one condition
  bool cond_entity(const Cond& c, u32 id, const T* planes, const unsigned char* cross, const T* boxes, T tol) const
  {
    if (c.kind == kCondFrustum)
    {
      for (u32 i = c.first; i < c.first + c.count; ++i)
      {
        const PlaneRel r = entity_plane(id, planes + 4 * i, tol);
        if (r == PlaneRel::Negative || (r == PlaneRel::Hit && !cross[i]))
          return false;
      }
      return true;
    }
    if (c.kind == kCondPlane)
    {
      const T ptol = c.tol < 0 ? base_tolerance<T>() : T(c.tol);
      return entity_plane(id, planes + 4 * c.first, ptol) == PlaneRel::Hit;
    }
    const T* r = boxes + 6 * u64(c.first);
    if (!isBox)
      return G::box_contains_point(r, ent(id), tol);
    return c.kind == kCondRangeInside ? G::contains_box_no_tol(r, ent(id)) : G::overlapped_strict(r, ent(id), tol);
  }

  // ot_query.h:864-1026 Query<And / Or>: a node is entered when its conditions pass (all, or any),
  // its entities are kept when theirs pass
  std::vector<u32> query(const Cond* conds, size_t nc, const T* planes, const unsigned char* cross, const T* boxes, bool orOp, T tol) const
  {
    std::vector<u32> found;
    dfs(
      [&](const Node& n) {
        bool pass = !orOp;
        for (size_t i = 0; i < nc; ++i)
        {
          const bool c = cond_node(conds[i], n, planes, boxes, tol);
          if (orOp && c)
          {
            pass = true;
            break;
          }
          if (!orOp && !c)
          {
            pass = false;
            break;
          }
        }
        if (!pass)
          return false;
        for (u32 id : n.entities)
        {
          bool ok = !orOp;
          for (size_t i = 0; i < nc; ++i)
          {
            const bool c = cond_entity(conds[i], id, planes, cross, boxes, tol);
            if (orOp && c)
            {
              ok = true;
              break;
            }
            if (!orOp && !c)
            {
              ok = false;
              break;
            }
          }
          if (ok)
            found.push_back(id);
        }
        return true;
      },
      root());
    if (countWork)
      work.ids += found.size();
    return found;
  }

  // ot_query.h:767-833 FrustumCulling (planes: np x {origoDistance, nx, ny, nz})
  std::vector<u32> frustum(const T* planes, size_t np, T tol) const
  {
    std::vector<u32> found;
    if (np == 0)
      return found;
    dfs(
      [&](const Node& n) {
        bool select = true;
        for (size_t i = 0; i < np; ++i)
        {
          const T* pl = planes + 4 * i;
          PlaneRel r = G::box_plane(node_min(n), node_size(n), pl[0], pl + 1, tol);
          if (r == PlaneRel::Hit)
          {
            select = true;
            break;
          }
          if (r == PlaneRel::Negative)
          {
            select = false;
            break;
          }
        }
        if (!select)
          return false;
        for (u32 id : n.entities)
        {
          bool neg = false;
          for (size_t i = 0; i < np && !neg; ++i)
          {
            const T* pl = planes + 4 * i;
            PlaneRel r;
            if (isBox)
            {
              const T* b = ent(id);
              T bsize[3] = { T(b[3] - b[0]), T(b[4] - b[1]), T(b[5] - b[2]) };
              r = G::box_plane(b, bsize, pl[0], pl + 1, tol);
            }
            else
              r = G::point_plane(ent(id), pl[0], pl + 1, tol);
            neg = (r == PlaneRel::Negative);
          }
          if (!neg)
            found.push_back(id);
        }
        return true;
      },
      root());
    return found;
  }

  // ot_query.h:235-291 TraverseNodesByPriority
  template<typename Proc, typename Prio>
  void traverse_by_priority(Proc&& proc, Prio&& prio) const
  {
    struct PN
    {
      const Node* node;
      T priority;
      auto operator<=>(const PN& o) const { return priority <=> o.priority; }
      bool operator==(const PN& o) const { return priority == o.priority; }
    };
    auto p0 = prio(root());
    if (!p0)
      return;
    std::priority_queue<PN, std::vector<PN>, std::greater<PN>> q;
    q.push({ &root(), *p0 });
    while (!q.empty())
    {
      auto [n, pr] = q.top();
      q.pop();
      int control = proc(*n, pr); // 0 continue, 1 skip children, 2 terminate
      if (control == 2)
        return;
      if (control == 1)
        continue;
      for (u64 ck : n->children)
      {
        const Node& c = nodes.at(ck);
        auto pc = prio(c);
        if (!pc)
          continue;
        q.push({ &c, *pc });
      }
    }
  }

  struct EntityDistance
  {
    u32 id;
    T distance;
    auto operator<=>(const EntityDistance& o) const { return distance <=> o.distance; }
    bool operator==(const EntityDistance& o) const { return distance == o.distance; }
  };

  // ot_query.h:1033-1036
  static T upper_tol(T v, T tol) { return std::fmax(tol, v * (T(1.0) + tol)); }

  // ot_query.h:1058-1164 AddEntityDistance
  void add_entity_distance(size_t k, const T* q, const std::vector<u32>& ids, T tol, std::vector<EntityDistance>& opt,
                           std::vector<EntityDistance>& pes, T& farthest) const
  {
    for (u32 id : ids)
    {
      T dmin, dminMax;
      if (!isBox)
      {
        T dist = G::distance(q, ent(id));
        dmin = dminMax = dist;
      }
      else
      {
        auto mm = G::min_max_distance(q, ent(id), tol);
        dmin = mm.first;
        dminMax = mm.second;
      }
      if (dmin >= farthest)
        continue;
      bool shouldHeapify = opt.size() == k - 1;
      opt.push_back({ id, dmin });
      pes.push_back({ id, dminMax });
      if (pes.size() < k)
        continue;
      if (shouldHeapify)
      {
        std::ranges::make_heap(opt);
        std::ranges::make_heap(pes);
        farthest = upper_tol(pes[0].distance, tol);
      }
      else
      {
        std::ranges::push_heap(opt);
        std::ranges::push_heap(pes);
        std::ranges::pop_heap(pes);
        pes.pop_back();
        T limit = upper_tol(pes.front().distance, tol);
        if (limit < farthest)
        {
          farthest = limit;
          bool removed = false;
          while (opt.front().distance > farthest)
          {
            u32 rid = opt.front().id;
            auto it = std::ranges::find_if(pes, [rid](const EntityDistance& ed) { return ed.id == rid; });
            if (it != pes.end())
            {
              pes.erase(it);
              removed = true;
            }
            std::ranges::pop_heap(opt);
            opt.pop_back();
          }
          if (removed)
            std::ranges::make_heap(pes);
        }
      }
    }
  }

  // ot_query.h:1208-1247 GetNearestNeighbors. Returns (id, distance) pairs in the reference's order.
  std::vector<EntityDistance> knn(const T* q, size_t k, T maxDistanceWithin, T tol) const
  {
    std::vector<EntityDistance> opt, pes;
    if (k == 0)
      return opt;
    T farthest = (maxDistanceWithin == std::numeric_limits<T>::max()) ? std::numeric_limits<T>::max() : upper_tol(maxDistanceWithin, tol);
    traverse_by_priority(
      [&](const Node& n, T nodeDistance) -> int {
        if (nodeDistance >= farthest)
          return 2;
        if (countWork)
          work.entities += n.entities.size();
        add_entity_distance(k, q, n.entities, tol, opt, pes, farthest);
        return 0;
      },
      [&](const Node& n) -> std::optional<T> {
        if (countWork)
          ++work.nodes;
        T w = G::wall_distance(q, node_min(n), node_size(n));
        if (w >= farthest)
          return std::nullopt;
        return w;
      });
    // ot_query.h:1166-1191 ConvertEntityDistanceToList
    if (countWork)
      work.ids += opt.size();
    if (opt.empty())
      return opt;
    if (opt.size() < k)
      std::sort(opt.begin(), opt.end());
    else
      std::sort_heap(opt.begin(), opt.end());
    return opt;
  }

  // ---------------------------------------------------------------- collision detection
  // ot_query.h:1274-1300 SweepAndPruneDatabase order: by min-x only (std::sort, unstable)
  std::vector<u32> sorted_by_minx(const std::vector<u32>& ids) const
  {
    std::vector<u32> s(ids);
    std::sort(s.begin(), s.end(), [&](u32 a, u32 b) { return ent(a)[0] < ent(b)[0]; });
    return s;
  }

  // ot_query.h:1308-1458 two-tree CollisionDetection (breadth-first node-pair queue)
  static void collide_trees(const Tree& L, const Node& lroot, const Tree& Rt, const Node& rroot, T tol, std::vector<std::pair<u32, u32>>& out)
  {
    struct NS
    {
      const Node* n;
      bool traversed;
    };
    std::unordered_map<const Node*, std::vector<u32>> cache[2];
    bool same = &L == &Rt;
    auto inOrder = [&](int side, const Node* n) -> const std::vector<u32>& {
      if (same)
        side = 0;
      const Tree& t = side == 0 ? L : Rt;
      auto it = cache[side].find(n);
      if (it == cache[side].end())
        it = cache[side].emplace(n, t.sorted_by_minx(n->entities)).first;
      return it->second;
    };
    std::queue<std::array<NS, 2>> q;
    q.push({ NS{ &lroot, false }, NS{ &rroot, false } });
    while (!q.empty())
    {
      auto pp = q.front();
      q.pop();
      const auto& le = inOrder(0, pp[0].n);
      const auto& re = inOrder(1, pp[1].n);
      size_t rn = re.size();
      size_t rb = 0;
      for (u32 lid : le)
      {
        const T* lg = L.ent(lid);
        for (; rb < rn; ++rb)
        {
          const T* rg = Rt.ent(re[rb]);
          if (L.isBox ? (rg[3] >= lg[0]) : (rg[0] >= lg[0]))
            break;
        }
        for (size_t ri = rb; ri < rn; ++ri)
        {
          u32 rid = re[ri];
          const T* rg = Rt.ent(rid);
          if (L.isBox)
          {
            if (lg[3] < rg[0])
              break;
            if (G::box_relation(lg, rg, tol) == -1)
              out.emplace_back(lid, rid);
          }
          else
          {
            if (lg[0] < rg[0])
              break;
            if (G::points_equal(lg, rg, tol))
              out.emplace_back(lid, rid);
          }
        }
      }
      std::array<std::vector<NS>, 2> ch;
      for (int s = 0; s < 2; ++s)
      {
        if (pp[s].traversed)
          continue;
        const Tree& t = s == 0 ? L : Rt;
        for (u64 ck : pp[s].n->children)
          ch[s].push_back({ &t.nodes.at(ck), false });
      }
      if (ch[0].empty() && ch[1].empty())
        continue;
      for (int s = 0; s < 2; ++s)
        if (!pp[s].n->entities.empty())
          ch[s].push_back({ pp[s].n, true });
      for (auto& lc : ch[0])
        for (auto& rc : ch[1])
          if (!(lc.n == pp[0].n && rc.n == pp[1].n))
            if (G::overlap_by_min_point(L.node_min(*lc.n), L.node_size(*lc.n), Rt.node_min(*rc.n), Rt.node_size(*rc.n), tol))
              q.push({ lc, rc });
    }
  }

  // ot_query.h:1500-1687 self collision, sequential path
  struct Ctx
  {
    const Node* n;
    T box[6];
    std::vector<u32> ids;
  };
  // ot_query.h:1699-1716 comparator: min-x, then id
  std::vector<u32> sorted_by_minx_id(const std::vector<u32>& ids) const
  {
    std::vector<u32> s(ids);
    std::sort(s.begin(), s.end(), [&](u32 a, u32 b) {
      T xa = ent(a)[0], xb = ent(b)[0];
      return xa < xb || (xa == xb && a < b);
    });
    return s;
  }
  void collide_subtree(const Node& n, std::vector<Ctx>& stack, T tol, std::vector<std::pair<u32, u32>>& out) const
  {
    Ctx c;
    c.n = &n;
    c.ids = sorted_by_minx_id(n.entities);
    node_box(n, c.box);
    stack.push_back(std::move(c));
    const Ctx& ctx = stack.back();
    // :1518-1561 inside node
    size_t m = ctx.ids.size();
    for (size_t i = 0; i < m; ++i)
    {
      const T* bi = ent(ctx.ids[i]);
      for (size_t j = i + 1; j < m; ++j)
      {
        const T* bj = ent(ctx.ids[j]);
        if (isBox)
        {
          if (bi[3] < bj[0])
            break;
          if (G::overlapped_strict(bi, bj, tol))
            out.emplace_back(ctx.ids[i], ctx.ids[j]);
        }
        else
        {
          if (bi[0] < bj[0])
            break;
          if (G::points_equal(bi, bj, tol))
            out.emplace_back(ctx.ids[i], ctx.ids[j]);
        }
      }
    }
    // :1563-1653 with parents
    const T* nmin = ctx.box;
    const T* nsize = node_size(n);
    for (size_t pd = 0; pd + 1 < stack.size(); ++pd)
    {
      const Ctx& par = stack[pd];
      size_t ib = 0;
      for (u32 pid : par.ids)
      {
        const T* pg = ent(pid);
        if (pg[0] > ctx.box[3])
          break;
        T pmin[3], psize[3];
        for (int d = 0; d < 3; ++d)
        {
          pmin[d] = pg[d];
          psize[d] = isBox ? T(pg[3 + d] - pg[d]) : T(0);
        }
        if (!G::overlap_by_min_point(nmin, nsize, pmin, psize, tol))
          continue;
        for (; ib < m; ++ib)
        {
          const T* eg = ent(ctx.ids[ib]);
          if (isBox ? (eg[3] >= pg[0]) : (eg[0] >= pg[0]))
            break;
        }
        for (size_t ie = ib; ie < m; ++ie)
        {
          u32 eid = ctx.ids[ie];
          const T* eg = ent(eid);
          if (isBox)
          {
            if (pg[3] < eg[0])
              break;
            if (G::overlapped_strict(eg, pg, tol))
              out.emplace_back(eid, pid);
          }
          else
          {
            if (pg[0] < eg[0])
              break;
            if (G::points_equal(pg, eg, tol))
              out.emplace_back(eid, pid);
          }
        }
      }
    }
    for (u64 ck : n.children)
      collide_subtree(nodes.at(ck), stack, tol, out);
    // :1672-1684 loose trees: pairwise sibling sub-trees
    if (loose)
    {
      for (size_t a = 0; a < n.children.size(); ++a)
        for (size_t b = a + 1; b < n.children.size(); ++b)
          collide_trees(*this, nodes.at(n.children[a]), *this, nodes.at(n.children[b]), tol, out);
    }
    stack.pop_back();
  }
  // ot_query.h:1690-1731, 1901-1906
  std::vector<std::pair<u32, u32>> collide_self(T tol) const
  {
    std::vector<std::pair<u32, u32>> out;
    std::vector<Ctx> stack;
    collide_subtree(root(), stack, tol, out);
    return out;
  }
  // ot_query.h:1462-1485
  static std::vector<std::pair<u32, u32>> collide_pair(const Tree& a, const Tree& b, T tol)
  {
    std::vector<std::pair<u32, u32>> out;
    collide_trees(a, a.root(), b, b.root(), tol, out);
    return out;
  }

  // ---------------------------------------------------------------- rays
  // ot_query.h:1928-2011 RayIntersectedAll (sorted by enter distance)
  std::vector<std::pair<u32, T>> ray_all(const T* o, const T* dir, T tol, T tolInc, T maxDist) const
  {
    std::vector<std::pair<u32, T>> found;
    auto rt = RayTester<T>::make(o, dir, tol, tolInc);
    if (!rt)
      return found;
    dfs(
      [&](const Node& n) {
        T en, ex;
        if (!rt->hit_node(node_min(n), node_size(n), en, ex))
          return false;
        for (u32 id : n.entities)
        {
          bool h = isBox ? rt->hit_box(ent(id), en, ex) : rt->hit_point(ent(id), en, ex);
          if (!h)
            continue;
          if (!(maxDist == 0 || en <= maxDist))
            continue;
          found.emplace_back(id, en);
        }
        return true;
      },
      root());
    std::sort(found.begin(), found.end(), [](auto& a, auto& b) { return a.second < b.second || (a.second == b.second && a.first < b.first); });
    return found;
  }

  // ot_query.h:2035-2122 RayIntersectedFirst (returned farthest first)
  std::vector<std::pair<u32, T>> ray_first(const T* o, const T* dir, T tol, T tolInc, T maxDistance) const
  {
    std::vector<std::pair<u32, T>> res;
    auto rt = RayTester<T>::make(o, dir, tol, tolInc);
    if (!rt)
      return res;
    struct Cand
    {
      u32 id;
      T enter;
      auto operator<=>(const Cand& o) const { return enter <=> o.enter; }
      bool operator==(const Cand& o) const { return enter == o.enter; }
    };
    T applied = tol == 0 ? std::numeric_limits<T>::epsilon() : tol;
    std::priority_queue<Cand, std::vector<Cand>> heap;
    T maxExam = maxDistance;
    traverse_by_priority(
      [&](const Node& n, T nodeEnter) -> int {
        if (nodeEnter > maxExam)
          return 2;
        for (u32 id : n.entities)
        {
          T en, ex;
          bool h = isBox ? rt->hit_box(ent(id), en, ex) : rt->hit_point(ent(id), en, ex);
          if (!h)
            continue;
          if (en > maxExam)
            continue;
          heap.push(Cand{ id, en });
          if (ex >= maxExam)
            continue;
          maxExam = (T(1) + tolInc) * ex + applied;
          while (!heap.empty() && heap.top().enter > maxExam)
            heap.pop();
        }
        return 0;
      },
      [&](const Node& n) -> std::optional<T> {
        T en, ex;
        if (!rt->hit_node(node_min(n), node_size(n), en, ex))
          return std::nullopt;
        return en;
      });
    for (; !heap.empty(); heap.pop())
      res.emplace_back(heap.top().id, heap.top().enter);
    return res;
  }
};

} // namespace otg_oracle
