// orthotree_gpu.hpp — C++20 drop-in types for OrthoTree's octrees (Core and Managed forms), backed
// by the GB300 library through its C-ABI (octree_gb300.h).
//
//   OrthoTreeGPU::OctreePoint    ~ OrthoTree::OctreePoint  (core/ot_aliases.h:119), Core: non-owning
//   OrthoTreeGPU::OctreeBox      ~ OrthoTree::OctreeBox    (core/ot_aliases.h:122), Core
//   OrthoTreeGPU::OctreeBoxs<L>  ~ OrthoTree::OctreeBoxs<L> (core/ot_aliases.h:144-145), Core
//   (and the FP32 Core variants OctreePointF / OctreeBoxF / OctreeBoxsF)
//   OrthoTreeGPU::OctreePointM   ~ OrthoTree::OctreePointM (core/ot_aliases.h:364)
//   OrthoTreeGPU::OctreeBoxM     ~ OrthoTree::OctreeBoxM   (core/ot_aliases.h:369)
//   OrthoTreeGPU::OctreeBoxMs<L> ~ OrthoTree::OctreeBoxMs<L> (core/ot_aliases.h:367-368; false: regular boxes)
//   (and the FP32 variants OctreePointMF / OctreeBoxMF / OctreeBoxMsF)
//
// The Core types take the entity span on Create and on every query, as the reference's do
// (core/ot_dynamic_hash_core.h:348-373, 812-822; core/ot_query.h:424-2146): the GPU keeps a device
// copy of the span it last saw and uploads another span (or the same one after
// NotifyEntitiesChanged) before a query, keeping the nodes, which is what the reference answers
// when it is given another span. The Managed types own their entities.
// Construction and Create take the reference's arguments (core/ot_managed.h:169-228, 318-360):
// entities, optional max depth, optional space box, max elements per node (default 16,
// core/configuration.h:83). Queries have the reference's names, argument order and defaults
// (core/ot_managed.h:584-893) and return the same id lists:
//   PickSearch, RangeSearch, FrustumCulling, PlaneSearch / PlaneIntersection,
//   PlanePositiveSegmentation, Query<And / Or> (ByWithin, ByOverlaps, ByInFrustum, ByIntersecting),
//   GetNearestNeighbors, RayIntersectedAll, RayIntersectedFirst, CollisionDetection (one tree and
//   two trees).
// Each query also has a batched form (…Batch) answering many query geometries in one GPU launch;
// it returns a Csr (offsets + ids [+ distances]). ExportStatic gives the arrays of the reference's
// static linear tree of the same entities; SaveStatic / LoadStatic write and resume its binary
// archive (serialization/binary_archive.h).
//
// Orders where the reference leaves ties unspecified are made canonical:
//   * GetNearestNeighbors and RayIntersectedAll: by (distance, id);
//   * RayIntersectedFirst: farthest first as the reference's max-heap pops them, ties by
//     descending id;
//   * CollisionDetection: pairs (i, j) ascending, i < j within one tree.
//
// Differences from the reference:
//   * Errors throw OrthoTreeGPU::Error, where the reference terminates (ORTHOTREE_CRASH_IF,
//     core/ot_base.h:104-108).
//   * The tester / callback overloads (TTester, FCollisionDetector, entityDistanceFn) and the
//     callback conditions of Query (BySatisfies) cannot run on the GPU and are not offered.
//   * Execution tags are accepted and ignored: the work runs on the GPU.
//   * There is no CPU fallback: without a CUDA device every call throws with status
//     OTG_ERR_NO_DEVICE.
#pragma once

#include "octree_gb300.h"

#include <array>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <optional>
#include <span>
#include <stdexcept>
#include <type_traits>
#include <unordered_set>
#include <string>
#include <utility>
#include <vector>

namespace OrthoTreeGPU
{
using index_t = std::uint32_t;
using EntityID = index_t;
using depth_t = std::uint32_t;

template<typename TScalar>
using Vector3 = std::array<TScalar, 3>;

// layouts of OrthoTree::BoundingBoxND / RayND / PlaneND (adapters/general.h:349-368)
template<typename TScalar>
struct BoundingBox3
{
  Vector3<TScalar> Min;
  Vector3<TScalar> Max;
};
template<typename TScalar>
struct Ray3
{
  Vector3<TScalar> Origin;
  Vector3<TScalar> Direction;
};
template<typename TScalar>
struct Plane3
{
  TScalar OrigoDistance;
  Vector3<TScalar> Normal;
};

using Point3D = Vector3<double>;
using BoundingBox3D = BoundingBox3<double>;
using Ray3D = Ray3<double>;
using Plane3D = Plane3<double>;

// core/types.h:83-87
enum class RangeSearchMode
{
  Inside = OTG_RANGE_INSIDE,
  Overlap = OTG_RANGE_OVERLAP
};

// core/types.h:69-73
enum class LogicalOperator
{
  And,
  Or
};

// query kernels: the default is the batched FP32-filtered kernel where one exists
enum class Algorithm
{
  Default = OTG_ALGO_DEFAULT,
  PlainFP64 = OTG_ALGO_PLAIN_FP64,
  Filtered = OTG_ALGO_FILTERED
};

class Error : public std::runtime_error
{
public:
  Error(int status, const std::string& what)
  : std::runtime_error(what)
  , m_status(status)
  {}
  int status() const noexcept { return m_status; }

private:
  int m_status;
};

// CSR result of a batched query: ids of query q are ids[offsets[q] .. offsets[q+1])
struct Csr
{
  std::vector<std::uint64_t> offsets;
  std::vector<EntityID> ids;
  std::vector<double> distances; // kNN and ray queries
  std::uint64_t filterTests = 0;
  std::uint64_t fp64Rechecks = 0;

  std::span<const EntityID> operator[](std::size_t q) const { return { ids.data() + offsets[q], ids.data() + offsets[q + 1] }; }
  std::size_t size() const { return offsets.empty() ? 0 : offsets.size() - 1; }
};

namespace detail
{
  inline void check(int rc)
  {
    if (rc != OTG_OK)
      throw Error(rc, std::string("octree_gb300: ") + otg_last_error());
  }

  template<typename TScalar>
  constexpr int scalar_code()
  {
    static_assert(std::is_same_v<TScalar, double> || std::is_same_v<TScalar, float>, "the GPU tree stores double or float");
    return std::is_same_v<TScalar, double> ? OTG_SCALAR_F64 : OTG_SCALAR_F32;
  }

  // the reference's BASE_TOLERANCE default (adapters/general.h:57): a negative value selects it
  template<typename TScalar>
  constexpr double base_tolerance()
  {
    return double(std::numeric_limits<TScalar>::epsilon()) * 100.0;
  }

  // maxDistance = numeric_limits::max() (the reference's "unbounded") maps to the C-ABI's < 0
  template<typename TScalar>
  inline double max_distance_arg(TScalar d)
  {
    return d == std::numeric_limits<TScalar>::max() ? -1.0 : double(d);
  }

  inline Csr take(otg_result* r, void* stream)
  {
    struct Guard
    {
      otg_result* r;
      ~Guard() { otg_result_free(r); }
    } g{ r };
    std::uint64_t nq = 0, n = 0;
    int hasDist = 0;
    check(otg_result_info(r, &nq, &n, &hasDist));
    Csr out;
    out.offsets.resize(nq + 1);
    out.ids.resize(n);
    if (hasDist)
      out.distances.resize(n);
    check(otg_result_copy(r, out.offsets.data(), out.ids.data(), hasDist ? out.distances.data() : nullptr, OTG_MEM_HOST, stream));
    check(otg_result_stats(r, &out.filterTests, &out.fp64Rechecks));
    return out;
  }

  inline std::vector<std::pair<EntityID, EntityID>> pairs_of(const Csr& c)
  {
    std::vector<std::pair<EntityID, EntityID>> p(c.ids.size() / 2);
    for (std::size_t i = 0; i < p.size(); ++i)
      p[i] = { c.ids[2 * i], c.ids[2 * i + 1] };
    return p;
  }
} // namespace detail

// Managed tree: owns a device copy of its entities (core/ot_managed.h:70-71).
template<typename TEntity, typename TScalar, int KIND>
class OrthoTreeManagedGPU
{
public:
  using Entity = TEntity;
  using TBox = BoundingBox3<TScalar>;
  using TVector = Vector3<TScalar>;
  using TRay = Ray3<TScalar>;
  using TPlane = Plane3<TScalar>;
  static constexpr std::size_t DEFAULT_TARGET_ELEMENT_NUM_IN_NODES = 16;

  OrthoTreeManagedGPU() { detail::check(otg_tree_new(&m_tree, detail::scalar_code<TScalar>(), KIND)); }

  // OrthoTreeManaged(geometryCollection, maxDepthID, boxSpace, maxElementNoInNode, execMode)
  template<typename TExecMode = std::nullptr_t>
  explicit OrthoTreeManagedGPU(std::span<const Entity> entities, std::optional<depth_t> maxDepthID = std::nullopt,
                               std::optional<TBox> boxSpace = std::nullopt, std::size_t maxElementNoInNode = DEFAULT_TARGET_ELEMENT_NUM_IN_NODES,
                               TExecMode = {})
  : OrthoTreeManagedGPU()
  {
    Create(entities, maxDepthID, boxSpace, maxElementNoInNode);
  }

  OrthoTreeManagedGPU(const OrthoTreeManagedGPU&) = delete;
  OrthoTreeManagedGPU& operator=(const OrthoTreeManagedGPU&) = delete;
  OrthoTreeManagedGPU(OrthoTreeManagedGPU&& o) noexcept
  : m_tree(std::exchange(o.m_tree, nullptr))
  , m_stream(o.m_stream)
  {}
  OrthoTreeManagedGPU& operator=(OrthoTreeManagedGPU&& o) noexcept
  {
    if (this != &o)
    {
      otg_tree_free(m_tree);
      m_tree = std::exchange(o.m_tree, nullptr);
      m_stream = o.m_stream;
    }
    return *this;
  }
  ~OrthoTreeManagedGPU() { otg_tree_free(m_tree); }

  // CUDA stream (cudaStream_t) the tree's work is ordered on; nullptr = legacy default stream
  void SetStream(void* stream) noexcept { m_stream = stream; }
  void* Stream() const noexcept { return m_stream; }
  const otg_tree* Handle() const noexcept { return m_tree; }

  // Create(entities, maxDepthID, boxSpace, maxElementNoInNode) — core/ot_dynamic_hash_core.h:751-822
  void Create(std::span<const Entity> entities, std::optional<depth_t> maxDepthID = std::nullopt, std::optional<TBox> boxSpace = std::nullopt,
              std::size_t maxElementNoInNode = DEFAULT_TARGET_ELEMENT_NUM_IN_NODES)
  {
    static_assert(sizeof(Entity) == sizeof(TScalar) * (KIND == OTG_KIND_POINTS ? 3 : 6), "entity layout");
    detail::check(otg_tree_create(m_tree, entities.data(), entities.size(), maxDepthID.value_or(0), boxSpace ? &*boxSpace : nullptr,
                                  maxElementNoInNode, OTG_MEM_HOST, m_stream));
  }

  // Add(newEntities, execMode): bulk Insert (core/ot_managed.h:421-455, which calls
  // DynamicHashOrthoTreeCore::Insert, core/ot_dynamic_hash_core.h:1012-1333). The new entities get the
  // ids GetEntityCount() .. GetEntityCount() + n - 1, as the reference numbers a contiguous span
  // (:1061-1064). false, and nothing added, when one lies outside the tree's space (the reference's
  // answer for non-keyed entities when out-of-space insertion is off; with it on, the reference
  // stores such a point with location code 0). Point trees.
  template<typename TExecMode = std::nullptr_t>
  bool Add(std::span<const Entity> newEntities, TExecMode = {})
    requires(KIND == OTG_KIND_POINTS)
  {
    const int rc = otg_tree_insert(m_tree, newEntities.data(), newEntities.size(), OTG_MEM_HOST, m_stream);
    if (rc == OTG_ERR_INVALID_ARGUMENT && newEntities.data())
      return false;
    detail::check(rc);
    return true;
  }
  std::size_t GetEntityCount() const { return std::size_t(Info().entity_count); }

  otg_tree_info Info() const
  {
    otg_tree_info info{};
    detail::check(otg_tree_info_get(m_tree, &info));
    return info;
  }
  std::size_t GetNodeCount() const { return std::size_t(Info().node_count); }
  depth_t GetMaxDepthID() const { return Info().max_depth; }

  // ---------------------------------------------------------------- static form and archives
  // The arrays of StaticLinearOrthoTreeCore (core/ot_static_linear_core.h:81-89, GetNodes(),
  // GetNodeDepthIDs(), GetEntityStorage(), GetNodeGeometries()) for these entities, computed on
  // the device: NodeStorageGeneral widths; geometry per node is the MinPoint (points) or
  // {minPoint, size} (boxes).
  struct StaticLayout
  {
    std::vector<std::uint32_t> nodeChildSegmentBegins; // as stored: up to the last node with children + 1
    std::vector<std::pair<std::uint32_t, std::uint32_t>> nodeEntitySegment; // {begin, length}
    std::vector<std::uint8_t> nodeDepthIDs;
    std::vector<EntityID> entityStorage;
    std::vector<TScalar> nodeGeometry; // 3 (points) or 6 (boxes) scalars per node
  };
  StaticLayout ExportStatic() const
  {
    otg_static_layout l{};
    detail::check(otg_tree_export_static(m_tree, &l, m_stream));
    StaticLayout s;
    std::vector<std::uint32_t> begins(l.node_count + 1), seg(2 * l.node_count);
    s.nodeDepthIDs.resize(l.node_count);
    s.entityStorage.resize(l.entity_count);
    s.nodeGeometry.resize(l.node_count * l.geometry_per_node);
    detail::check(otg_static_layout_copy(&l, l.node_count ? begins.data() : nullptr, seg.data(), s.nodeDepthIDs.data(), s.entityStorage.data(),
                                         s.nodeGeometry.data()));
    s.nodeChildSegmentBegins.assign(begins.begin(), begins.begin() + l.child_begin_count);
    for (std::size_t i = 0; i < l.node_count; ++i)
      s.nodeEntitySegment.emplace_back(seg[2 * i], seg[2 * i + 1]);
    return s;
  }

  // `ar & tree` of the reference's BinaryOutputArchive for StaticOctreePointM / StaticOctreeBoxM
  // (withEntities) or StaticOctreePoint / StaticOctreeBox (serialization.h:359-385, 433-438)
  std::vector<std::uint8_t> SaveStatic(bool withEntities = true) const
  {
    std::uint64_t size = 0;
    detail::check(otg_tree_save_static(m_tree, withEntities ? 1 : 0, nullptr, 0, &size, m_stream));
    std::vector<std::uint8_t> bytes(size);
    detail::check(otg_tree_save_static(m_tree, withEntities ? 1 : 0, bytes.data(), size, &size, m_stream));
    return bytes;
  }

  // Resumes from a Managed archive (the reference's or SaveStatic's): rebuilds its entities in
  // boxSpace (default: their bounding box) and checks the rebuild against the archive
  void LoadStatic(std::span<const std::uint8_t> archive, std::optional<TBox> boxSpace = std::nullopt)
  {
    detail::check(otg_tree_load_static(m_tree, archive.data(), archive.size(), boxSpace ? &*boxSpace : nullptr, m_stream));
  }

  // ---------------------------------------------------------------- single queries (reference form)
  std::vector<EntityID> PickSearch(const TVector& pickPoint, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return first(PickSearchBatch(std::span<const TVector>(&pickPoint, 1), tolerance));
  }

  std::vector<EntityID> RangeSearch(const TBox& range, RangeSearchMode mode = RangeSearchMode::Inside,
                                    double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return first(RangeSearchBatch(std::span<const TBox>(&range, 1), mode, tolerance));
  }

  std::vector<EntityID> FrustumCulling(std::span<const TPlane> boundaryPlanes, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return first(FrustumCullingBatch(boundaryPlanes, boundaryPlanes.size(), tolerance));
  }

  // core/ot_query.h:612-664 (PlaneSearch; PlaneIntersection is the same query)
  std::vector<EntityID> PlaneSearch(TScalar distanceOfOrigo, const TVector& planeNormal, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    const TPlane plane{ distanceOfOrigo, planeNormal };
    return first(PlaneSearchBatch(std::span<const TPlane>(&plane, 1), tolerance));
  }
  std::vector<EntityID> PlaneSearch(const TPlane& plane, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return first(PlaneSearchBatch(std::span<const TPlane>(&plane, 1), tolerance));
  }
  std::vector<EntityID> PlaneIntersection(const TPlane& plane, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return PlaneSearch(plane, tolerance);
  }
  // core/ot_query.h:687-758
  std::vector<EntityID> PlanePositiveSegmentation(TScalar distanceOfOrigo, const TVector& planeNormal,
                                                  double tolerance = detail::base_tolerance<TScalar>()) const
  {
    const TPlane plane{ distanceOfOrigo, planeNormal };
    return first(PlanePositiveSegmentationBatch(std::span<const TPlane>(&plane, 1), tolerance));
  }
  std::vector<EntityID> PlanePositiveSegmentation(const TPlane& plane, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return first(PlanePositiveSegmentationBatch(std::span<const TPlane>(&plane, 1), tolerance));
  }

  // core/ot_query.h:835-861: one condition of Query (the callback conditions are not offered)
  struct QueryCondition
  {
    int kind = OTG_COND_RANGE_INSIDE;
    std::vector<std::pair<TPlane, bool>> planes; // frustum: planes with isCrossingAllowed; plane condition: its plane
    TBox range{};
    double tolerance = -1.0;                     // plane condition: its own tolerance
  };
  static QueryCondition ByWithin(const TBox& range) { return { OTG_COND_RANGE_INSIDE, {}, range, -1.0 }; }
  static QueryCondition ByOverlaps(const TBox& range) { return { OTG_COND_RANGE_OVERLAP, {}, range, -1.0 }; }
  static QueryCondition ByInFrustum(std::vector<std::pair<TPlane, bool>> boundaryPlanes)
  {
    return { OTG_COND_FRUSTUM, std::move(boundaryPlanes), {}, -1.0 };
  }
  static QueryCondition ByIntersecting(const TPlane& plane, double tolerance = detail::base_tolerance<TScalar>())
  {
    return { OTG_COND_PLANE, { { plane, false } }, {}, tolerance };
  }

  // core/ot_query.h:864-1026 Query<And / Or>(conditions, entities, tolerance)
  template<LogicalOperator OP = LogicalOperator::And, typename TConditions>
  std::vector<EntityID> Query(const TConditions& conditions, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    const std::vector<std::vector<QueryCondition>> one(1, std::vector<QueryCondition>(std::begin(conditions), std::end(conditions)));
    return first(QueryBatch<OP>(one, tolerance));
  }

  std::vector<EntityID> GetNearestNeighbors(const TVector& searchPoint, std::size_t neighborCount, TScalar maxDistanceWithin,
                                            double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return first(GetNearestNeighborsBatch(std::span<const TVector>(&searchPoint, 1), neighborCount, maxDistanceWithin, tolerance));
  }
  std::vector<EntityID> GetNearestNeighbors(const TVector& searchPoint, std::size_t neighborCount, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return GetNearestNeighbors(searchPoint, neighborCount, std::numeric_limits<TScalar>::max(), tolerance);
  }

  std::vector<EntityID> RayIntersectedAll(const TVector& rayBasePoint, const TVector& rayHeading, double tolerance = detail::base_tolerance<TScalar>(),
                                          double toleranceIncrement = 0.0, TScalar maxExaminationDistance = std::numeric_limits<TScalar>::max()) const
  {
    const TRay ray{ rayBasePoint, rayHeading };
    return first(RayIntersectedAllBatch(std::span<const TRay>(&ray, 1), tolerance, toleranceIncrement, maxExaminationDistance));
  }
  std::vector<EntityID> RayIntersectedAll(const TRay& ray, double tolerance = detail::base_tolerance<TScalar>(), double toleranceIncrement = 0.0,
                                          TScalar maxExaminationDistance = std::numeric_limits<TScalar>::max()) const
  {
    return RayIntersectedAll(ray.Origin, ray.Direction, tolerance, toleranceIncrement, maxExaminationDistance);
  }

  std::vector<EntityID> RayIntersectedFirst(const TVector& rayBasePoint, const TVector& rayHeading, double tolerance = detail::base_tolerance<TScalar>(),
                                            double toleranceIncrement = 0.0, TScalar maxDistance = std::numeric_limits<TScalar>::max()) const
  {
    const TRay ray{ rayBasePoint, rayHeading };
    auto ids = first(RayIntersectedFirstBatch(std::span<const TRay>(&ray, 1), tolerance, toleranceIncrement, maxDistance));
    return { ids.rbegin(), ids.rend() }; // the reference's max-heap pops the farthest first
  }
  std::vector<EntityID> RayIntersectedFirst(const TRay& ray, double tolerance = detail::base_tolerance<TScalar>(), double toleranceIncrement = 0.0,
                                            TScalar maxDistance = std::numeric_limits<TScalar>::max()) const
  {
    return RayIntersectedFirst(ray.Origin, ray.Direction, tolerance, toleranceIncrement, maxDistance);
  }

  // ---------------------------------------------------------------- batched queries (one launch)
  Csr PickSearchBatch(std::span<const TVector> points, double tolerance = detail::base_tolerance<TScalar>(), Algorithm algo = Algorithm::Default) const
  {
    otg_result* r = nullptr;
    detail::check(otg_pick_search(m_tree, points.data(), points.size(), tolerance, int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  Csr RangeSearchBatch(std::span<const TBox> ranges, RangeSearchMode mode = RangeSearchMode::Inside, double tolerance = detail::base_tolerance<TScalar>(),
                       Algorithm algo = Algorithm::Default) const
  {
    otg_result* r = nullptr;
    detail::check(otg_range_search(m_tree, ranges.data(), ranges.size(), int(mode), tolerance, int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  // planes: n_queries consecutive groups of planesPerQuery planes
  Csr FrustumCullingBatch(std::span<const TPlane> planes, std::size_t planesPerQuery, double tolerance = detail::base_tolerance<TScalar>(),
                          Algorithm algo = Algorithm::Default) const
  {
    if (planesPerQuery == 0 || planes.size() % planesPerQuery)
      throw Error(OTG_ERR_INVALID_ARGUMENT, "planes must hold whole groups of planesPerQuery");
    otg_result* r = nullptr;
    detail::check(otg_frustum_culling(m_tree, planes.data(), planesPerQuery, planes.size() / planesPerQuery, tolerance, int(algo), &r, OTG_MEM_HOST,
                                      m_stream));
    return detail::take(r, m_stream);
  }
  // one plane per query
  Csr PlaneSearchBatch(std::span<const TPlane> planes, double tolerance = detail::base_tolerance<TScalar>(), Algorithm algo = Algorithm::Default) const
  {
    otg_result* r = nullptr;
    detail::check(otg_plane_search(m_tree, planes.data(), planes.size(), tolerance, int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  Csr PlanePositiveSegmentationBatch(std::span<const TPlane> planes, double tolerance = detail::base_tolerance<TScalar>(),
                                     Algorithm algo = Algorithm::Default) const
  {
    otg_result* r = nullptr;
    detail::check(otg_plane_positive_segmentation(m_tree, planes.data(), planes.size(), tolerance, int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  // one condition list per query
  template<LogicalOperator OP = LogicalOperator::And>
  Csr QueryBatch(std::span<const std::vector<QueryCondition>> queries, double tolerance = detail::base_tolerance<TScalar>(),
                 Algorithm algo = Algorithm::Default) const
  {
    std::vector<otg_condition> conds;
    std::vector<std::uint64_t> offsets{ 0 };
    std::vector<TPlane> planes;
    std::vector<std::uint8_t> crossing;
    std::vector<TBox> boxes;
    for (const auto& q : queries)
    {
      for (const auto& c : q)
      {
        otg_condition oc{ c.kind, 0, 1, 0, c.tolerance };
        if (c.kind == OTG_COND_FRUSTUM || c.kind == OTG_COND_PLANE)
        {
          if (c.kind == OTG_COND_PLANE && c.planes.size() != 1)
            throw Error(OTG_ERR_INVALID_ARGUMENT, "a plane condition holds one plane");
          oc.first = std::uint32_t(planes.size());
          oc.count = std::uint32_t(c.planes.size());
          for (const auto& [plane, crossingAllowed] : c.planes)
          {
            planes.push_back(plane);
            crossing.push_back(crossingAllowed ? 1 : 0);
          }
        }
        else
        {
          oc.first = std::uint32_t(boxes.size());
          boxes.push_back(c.range);
        }
        conds.push_back(oc);
      }
      offsets.push_back(conds.size());
    }
    otg_result* r = nullptr;
    detail::check(otg_query(m_tree, conds.data(), offsets.data(), queries.size(), planes.data(), crossing.data(), planes.size(), boxes.data(),
                            boxes.size(), OP == LogicalOperator::Or ? 1 : 0, tolerance, int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  Csr GetNearestNeighborsBatch(std::span<const TVector> points, std::size_t neighborCount,
                               TScalar maxDistanceWithin = std::numeric_limits<TScalar>::max(), double tolerance = detail::base_tolerance<TScalar>(),
                               Algorithm algo = Algorithm::Default) const
  {
    otg_result* r = nullptr;
    detail::check(otg_knn(m_tree, points.data(), points.size(), nullptr, std::uint32_t(neighborCount), detail::max_distance_arg(maxDistanceWithin),
                          tolerance, int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  // per-query neighbour counts
  Csr GetNearestNeighborsBatch(std::span<const TVector> points, std::span<const std::uint32_t> neighborCounts,
                               TScalar maxDistanceWithin = std::numeric_limits<TScalar>::max(), double tolerance = detail::base_tolerance<TScalar>(),
                               Algorithm algo = Algorithm::Default) const
  {
    if (neighborCounts.size() != points.size())
      throw Error(OTG_ERR_INVALID_ARGUMENT, "one neighbour count per query point");
    otg_result* r = nullptr;
    detail::check(otg_knn(m_tree, points.data(), points.size(), neighborCounts.data(), 0, detail::max_distance_arg(maxDistanceWithin), tolerance,
                          int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  Csr RayIntersectedAllBatch(std::span<const TRay> rays, double tolerance = detail::base_tolerance<TScalar>(), double toleranceIncrement = 0.0,
                             TScalar maxExaminationDistance = std::numeric_limits<TScalar>::max(), Algorithm algo = Algorithm::Default) const
  {
    otg_result* r = nullptr;
    detail::check(otg_ray_all(m_tree, rays.data(), rays.size(), tolerance, toleranceIncrement, detail::max_distance_arg(maxExaminationDistance),
                              int(algo), &r, OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }
  // ids per ray by (enter distance, id); RayIntersectedFirst() returns them farthest first
  Csr RayIntersectedFirstBatch(std::span<const TRay> rays, double tolerance = detail::base_tolerance<TScalar>(), double toleranceIncrement = 0.0,
                               TScalar maxDistance = std::numeric_limits<TScalar>::max(), Algorithm algo = Algorithm::Default) const
  {
    otg_result* r = nullptr;
    detail::check(otg_ray_first(m_tree, rays.data(), rays.size(), tolerance, toleranceIncrement, detail::max_distance_arg(maxDistance), int(algo), &r,
                                OTG_MEM_HOST, m_stream));
    return detail::take(r, m_stream);
  }

  // ---------------------------------------------------------------- collision (box trees)
  // CollisionDetection(tolerance, execMode) — core/ot_managed.h:700-709, core/ot_query.h:1902-1906
  template<typename TExecMode = std::nullptr_t>
  std::vector<std::pair<EntityID, EntityID>> CollisionDetection(double tolerance = detail::base_tolerance<TScalar>(), TExecMode = {},
                                                                Algorithm algo = Algorithm::Default) const
    requires(KIND != OTG_KIND_POINTS)
  {
    otg_result* r = nullptr;
    detail::check(otg_collision_self(m_tree, tolerance, int(algo), &r, m_stream));
    return detail::pairs_of(detail::take(r, m_stream));
  }
  // CollisionDetection(otherTree, tolerance) — core/ot_managed.h:712-718, core/ot_query.h:1462-1497
  std::vector<std::pair<EntityID, EntityID>> CollisionDetection(const OrthoTreeManagedGPU& otherTree, double tolerance = detail::base_tolerance<TScalar>(),
                                                                Algorithm algo = Algorithm::Default) const
    requires(KIND != OTG_KIND_POINTS)
  {
    otg_result* r = nullptr;
    detail::check(otg_collision_pair(m_tree, otherTree.m_tree, tolerance, int(algo), &r, m_stream));
    return detail::pairs_of(detail::take(r, m_stream));
  }
  static std::vector<std::pair<EntityID, EntityID>> CollisionDetection(const OrthoTreeManagedGPU& leftTree, const OrthoTreeManagedGPU& rightTree,
                                                                       double tolerance = detail::base_tolerance<TScalar>())
    requires(KIND != OTG_KIND_POINTS)
  {
    return leftTree.CollisionDetection(rightTree, tolerance);
  }

private:
  static std::vector<EntityID> first(const Csr& c) { return c.size() ? std::vector<EntityID>(c[0].begin(), c[0].end()) : std::vector<EntityID>{}; }

  otg_tree* m_tree = nullptr;
  void* m_stream = nullptr;
};

using OctreePointM = OrthoTreeManagedGPU<Vector3<double>, double, OTG_KIND_POINTS>;
using OctreeBoxM = OrthoTreeManagedGPU<BoundingBox3<double>, double, OTG_KIND_BOXES>;
using OctreePointMF = OrthoTreeManagedGPU<Vector3<float>, float, OTG_KIND_POINTS>;
using OctreeBoxMF = OrthoTreeManagedGPU<BoundingBox3<float>, float, OTG_KIND_BOXES>;
// OctreeBoxMs<IS_LOOSE_TREE> (core/ot_aliases.h:367-368): false = the regular box tree (loose factor 1.0)
template<bool IS_LOOSE_TREE>
using OctreeBoxMs = OrthoTreeManagedGPU<BoundingBox3<double>, double, IS_LOOSE_TREE ? OTG_KIND_BOXES : OTG_KIND_BOXES_REGULAR>;
template<bool IS_LOOSE_TREE>
using OctreeBoxMsF = OrthoTreeManagedGPU<BoundingBox3<float>, float, IS_LOOSE_TREE ? OTG_KIND_BOXES : OTG_KIND_BOXES_REGULAR>;

// Core tree: non-owning, as OrthoTree's Core types (OctreePoint, OctreeBox, OctreeBoxs<L>;
// core/ot_aliases.h:119-145). Create takes the entities, and so does every query
// (EntityContainerView = std::span<T const>, core/entity_adapter.h:171-174); the reference tests
// the geometry of the span it is given against the nodes Create built
// (core/ot_dynamic_hash_core.h:812-822, core/ot_query.h:424-427, 477-482, 1209-1215, 1902-1906).
// The GPU needs that geometry in device memory, so the tree keeps a device copy of the span it
// last saw, identified by (pointer, size, generation). A query with the same span and generation
// uses the device copy as it is. A query with another span, or after NotifyEntitiesChanged() (the
// caller changed the span's contents in place), uploads that span first, by the tree's SpanChange
// policy:
//   * Rebuild (default): the tree is created again from the new span with the arguments of the last
//     Create, so every query answers as the reference's tree of that span does. The reference
//     instead keeps the nodes it built from the earlier span.
//   * KeepNodes: the nodes stay and only the tested geometry changes (otg_tree_set_entities), as the
//     reference does; a span of another size is refused (OTG_ERR_INVALID_ARGUMENT). Where
//     entities moved outside the nodes they were built into, the reference's kNN,
//     RayIntersectedFirst and collision answers depend on the order of its own traversal, and the
//     GPU's may differ from them; RangeSearch, PickSearch, FrustumCulling, the plane queries, Query
//     and RayIntersectedAll test a fixed set of nodes and entities and answer as the reference does.
// The check makes queries on one tree object unsafe to call concurrently with different spans.
template<typename TEntity, typename TScalar, int KIND>
class OrthoTreeCoreGPU
{
  using Impl = OrthoTreeManagedGPU<TEntity, TScalar, KIND>;

public:
  using Entity = TEntity;
  using EntityContainerView = std::span<const TEntity>;
  using TBox = typename Impl::TBox;
  using TVector = typename Impl::TVector;
  using TRay = typename Impl::TRay;
  using TPlane = typename Impl::TPlane;
  using QueryCondition = typename Impl::QueryCondition;
  static constexpr std::size_t DEFAULT_TARGET_ELEMENT_NUM_IN_NODES = Impl::DEFAULT_TARGET_ELEMENT_NUM_IN_NODES;

  enum class SpanChange
  {
    Rebuild,
    KeepNodes
  };

  OrthoTreeCoreGPU() = default;

  // DynamicHashOrthoTreeCore(entities, maxDepthID, boxSpace, maxElementNoInNode, execMode) (:348-358)
  template<typename TExecMode = std::nullptr_t>
  explicit OrthoTreeCoreGPU(EntityContainerView entities, std::optional<depth_t> maxDepthID = std::nullopt, std::optional<TBox> boxSpace = std::nullopt,
                            std::size_t maxElementNoInNode = DEFAULT_TARGET_ELEMENT_NUM_IN_NODES, TExecMode = {})
  {
    Create(entities, maxDepthID, boxSpace, maxElementNoInNode);
  }
  // DynamicHashOrthoTreeCore(execMode, entities, maxDepthID, boxSpace, maxElementNoInNode) (:362-373)
  template<typename TExecMode>
    requires(!std::is_convertible_v<TExecMode, EntityContainerView>)
  OrthoTreeCoreGPU(TExecMode, EntityContainerView entities, std::optional<depth_t> maxDepthID = std::nullopt, std::optional<TBox> boxSpace = std::nullopt,
                   std::size_t maxElementNoInNode = DEFAULT_TARGET_ELEMENT_NUM_IN_NODES)
  {
    Create(entities, maxDepthID, boxSpace, maxElementNoInNode);
  }

  void SetStream(void* stream) noexcept { m_impl.SetStream(stream); }
  const otg_tree* Handle() const noexcept { return m_impl.Handle(); }

  // Create(entities, maxDepthID, boxSpace, maxElementNoInNode, execMode) (:751-809); errors throw
  template<typename TExecMode = std::nullptr_t>
  bool Create(EntityContainerView entities, std::optional<depth_t> maxDepthID = std::nullopt, std::optional<TBox> boxSpace = std::nullopt,
              std::size_t maxElementNoInNode = DEFAULT_TARGET_ELEMENT_NUM_IN_NODES, TExecMode = {})
  {
    m_impl.Create(entities, maxDepthID, boxSpace, maxElementNoInNode);
    m_maxDepth = maxDepthID;
    m_box = boxSpace;
    m_maxElem = maxElementNoInNode;
    m_data = entities.data();
    m_size = entities.size();
    m_boundGeneration = m_generation;
    return true;
  }
  // static Create(tree, entities, maxDepthID, boxSpace, maxElementNoInNode, execMode) (:812-822)
  template<typename TExecMode = std::nullptr_t>
  static bool Create(OrthoTreeCoreGPU& tree, EntityContainerView entities, std::optional<depth_t> maxDepthID = std::nullopt,
                     std::optional<TBox> boxSpace = std::nullopt, std::size_t maxElementNoInNode = DEFAULT_TARGET_ELEMENT_NUM_IN_NODES, TExecMode = {})
  {
    return tree.Create(entities, maxDepthID, boxSpace, maxElementNoInNode);
  }

  // Insert(newEntities, existingEntities, execMode, failedEntities) (core/ot_dynamic_hash_core.h:
  // 1012-1333): bulk Insert of points with the ids existingEntities.size() + i (:1061-1064);
  // existingEntities is the span the tree was built for (its size is the tree's entity count). The
  // next query's span of the grown size (existing then new entities, as the caller appends them)
  // is taken as the tree's geometry without a rebuild. false, nothing inserted and the ids of the
  // points outside the tree's space in failedEntities, when any lies outside it.
  template<typename TExecMode = std::nullptr_t>
  bool Insert(EntityContainerView newEntities, EntityContainerView existingEntities, TExecMode = {},
              std::unordered_set<EntityID>* failedEntities = nullptr)
    requires(KIND == OTG_KIND_POINTS)
  {
    const std::size_t n = m_impl.GetEntityCount();
    if (existingEntities.size() != n)
      throw Error(OTG_ERR_INVALID_ARGUMENT, "Insert: existingEntities must be the span the tree holds");
    if (!m_impl.Add(newEntities))
    {
      if (failedEntities)
      {
        const otg_tree_info info = m_impl.Info();
        for (std::size_t i = 0; i < newEntities.size(); ++i)
        {
          bool in = true;
          for (int d = 0; d < 3; ++d)
          {
            const double v = double(newEntities[i][d]);
            in = in && v >= info.space_min[d] && v <= info.space_max[d];
          }
          if (!in)
            failedEntities->insert(EntityID(n + i));
        }
      }
      return false;
    }
    m_data = nullptr;
    m_size = n + newEntities.size();
    m_grown = true;
    return true;
  }

  // The caller changed the contents of the span in place: the next query uploads it again.
  void NotifyEntitiesChanged() noexcept { ++m_generation; }
  void SetSpanChange(SpanChange policy) noexcept { m_policy = policy; }

  std::size_t GetNodeCount() const { return m_impl.GetNodeCount(); }
  depth_t GetMaxDepthID() const { return m_impl.GetMaxDepthID(); }

  // ---------------------------------------------------------------- queries (reference form)
  std::vector<EntityID> PickSearch(const TVector& pickPoint, EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).PickSearch(pickPoint, tolerance);
  }
  std::vector<EntityID> RangeSearch(const TBox& range, EntityContainerView entities, RangeSearchMode mode = RangeSearchMode::Inside,
                                    double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).RangeSearch(range, mode, tolerance);
  }
  std::vector<EntityID> PlaneSearch(TScalar distanceOfOrigo, const TVector& planeNormal, EntityContainerView entities,
                                    double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).PlaneSearch(distanceOfOrigo, planeNormal, tolerance);
  }
  std::vector<EntityID> PlaneSearch(const TPlane& plane, EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).PlaneSearch(plane, tolerance);
  }
  std::vector<EntityID> PlaneIntersection(TScalar distanceOfOrigo, const TVector& planeNormal, EntityContainerView entities,
                                          double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return PlaneSearch(distanceOfOrigo, planeNormal, entities, tolerance);
  }
  std::vector<EntityID> PlaneIntersection(const TPlane& plane, EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return PlaneSearch(plane, entities, tolerance);
  }
  std::vector<EntityID> PlanePositiveSegmentation(TScalar distanceOfOrigo, const TVector& planeNormal, EntityContainerView entities,
                                                  double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).PlanePositiveSegmentation(distanceOfOrigo, planeNormal, tolerance);
  }
  std::vector<EntityID> PlanePositiveSegmentation(const TPlane& plane, EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).PlanePositiveSegmentation(plane, tolerance);
  }
  std::vector<EntityID> FrustumCulling(std::span<const TPlane> boundaryPlanes, EntityContainerView entities,
                                       double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).FrustumCulling(boundaryPlanes, tolerance);
  }
  static QueryCondition ByWithin(const TBox& range) { return Impl::ByWithin(range); }
  static QueryCondition ByOverlaps(const TBox& range) { return Impl::ByOverlaps(range); }
  static QueryCondition ByInFrustum(std::vector<std::pair<TPlane, bool>> boundaryPlanes) { return Impl::ByInFrustum(std::move(boundaryPlanes)); }
  static QueryCondition ByIntersecting(const TPlane& plane, double tolerance = detail::base_tolerance<TScalar>())
  {
    return Impl::ByIntersecting(plane, tolerance);
  }
  template<LogicalOperator OP = LogicalOperator::And, typename TConditions>
  std::vector<EntityID> Query(const TConditions& conditions, EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).template Query<OP>(conditions, tolerance);
  }
  std::vector<EntityID> GetNearestNeighbors(const TVector& searchPoint, std::size_t neighborCount, TScalar maxDistanceWithin, EntityContainerView entities,
                                            double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).GetNearestNeighbors(searchPoint, neighborCount, maxDistanceWithin, tolerance);
  }
  std::vector<EntityID> GetNearestNeighbors(const TVector& searchPoint, std::size_t neighborNo, EntityContainerView entities,
                                            double tolerance = detail::base_tolerance<TScalar>()) const
  {
    return bind(entities).GetNearestNeighbors(searchPoint, neighborNo, std::numeric_limits<TScalar>::max(), tolerance);
  }
  std::vector<EntityID> RayIntersectedAll(const TVector& rayBasePoint, const TVector& rayHeading, EntityContainerView entities,
                                          double tolerance = detail::base_tolerance<TScalar>(), double toleranceIncrement = 0.0,
                                          TScalar maxExaminationDistance = std::numeric_limits<TScalar>::max()) const
  {
    return bind(entities).RayIntersectedAll(rayBasePoint, rayHeading, tolerance, toleranceIncrement, maxExaminationDistance);
  }
  std::vector<EntityID> RayIntersectedAll(const TRay& ray, EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>(),
                                          double toleranceIncrement = 0.0, TScalar maxExaminationDistance = std::numeric_limits<TScalar>::max()) const
  {
    return bind(entities).RayIntersectedAll(ray, tolerance, toleranceIncrement, maxExaminationDistance);
  }
  std::vector<EntityID> RayIntersectedFirst(const TVector& rayBasePoint, const TVector& rayHeading, EntityContainerView entities,
                                            double tolerance = detail::base_tolerance<TScalar>(), double toleranceIncrement = 0.0,
                                            TScalar maxDistance = std::numeric_limits<TScalar>::max()) const
  {
    return bind(entities).RayIntersectedFirst(rayBasePoint, rayHeading, tolerance, toleranceIncrement, maxDistance);
  }
  std::vector<EntityID> RayIntersectedFirst(const TRay& ray, EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>(),
                                            double toleranceIncrement = 0.0, TScalar maxDistance = std::numeric_limits<TScalar>::max()) const
  {
    return bind(entities).RayIntersectedFirst(ray, tolerance, toleranceIncrement, maxDistance);
  }

  // CollisionDetection(entities, tolerance, execMode) (core/ot_query.h:1902-1906)
  template<typename TExecMode = std::nullptr_t>
  std::vector<std::pair<EntityID, EntityID>> CollisionDetection(EntityContainerView entities, double tolerance = detail::base_tolerance<TScalar>(),
                                                                TExecMode = {}) const
    requires(KIND != OTG_KIND_POINTS)
  {
    return bind(entities).CollisionDetection(tolerance);
  }
  // CollisionDetection(entities, otherTree, otherEntities, tolerance) (core/ot_query.h:1489-1497)
  std::vector<std::pair<EntityID, EntityID>> CollisionDetection(EntityContainerView entities, const OrthoTreeCoreGPU& otherTree,
                                                                EntityContainerView otherEntities, double tolerance = detail::base_tolerance<TScalar>()) const
    requires(KIND != OTG_KIND_POINTS)
  {
    const Impl& left = bind(entities);
    return left.CollisionDetection(otherTree.bind(otherEntities), tolerance);
  }
  // static CollisionDetection(leftTree, leftEntities, rightTree, rightEntities, tolerance) (:1462-1485)
  static std::vector<std::pair<EntityID, EntityID>> CollisionDetection(const OrthoTreeCoreGPU& leftTree, EntityContainerView leftEntities,
                                                                       const OrthoTreeCoreGPU& rightTree, EntityContainerView rightEntities,
                                                                       double tolerance = detail::base_tolerance<TScalar>())
    requires(KIND != OTG_KIND_POINTS)
  {
    return leftTree.CollisionDetection(leftEntities, rightTree, rightEntities, tolerance);
  }

private:
  // the Managed tree behind the Core interface, its device entities made to be `entities`
  const Impl& bind(EntityContainerView entities) const
  {
    if (entities.data() != m_data || entities.size() != m_size || m_boundGeneration != m_generation)
    {
      // after an Insert the grown span (the old entities, then the new ones) is the tree's geometry
      const bool grown = m_grown && entities.size() == m_size;
      m_grown = false;
      if (m_policy == SpanChange::Rebuild && !grown)
        const_cast<Impl&>(m_impl).Create(entities, m_maxDepth, m_box, m_maxElem);
      else
        detail::check(otg_tree_set_entities(const_cast<otg_tree*>(m_impl.Handle()), entities.data(), entities.size(), OTG_MEM_HOST, m_impl.Stream()));
      m_data = entities.data();
      m_size = entities.size();
      m_boundGeneration = m_generation;
    }
    return m_impl;
  }

  Impl m_impl;
  std::optional<depth_t> m_maxDepth;
  std::optional<TBox> m_box;
  std::size_t m_maxElem = DEFAULT_TARGET_ELEMENT_NUM_IN_NODES;
  SpanChange m_policy = SpanChange::Rebuild;
  mutable const TEntity* m_data = nullptr;
  mutable std::size_t m_size = 0;
  std::uint64_t m_generation = 0;
  mutable std::uint64_t m_boundGeneration = 0;
  mutable bool m_grown = false;
};

using OctreePoint = OrthoTreeCoreGPU<Vector3<double>, double, OTG_KIND_POINTS>;
using OctreeBox = OrthoTreeCoreGPU<BoundingBox3<double>, double, OTG_KIND_BOXES>;
using OctreePointF = OrthoTreeCoreGPU<Vector3<float>, float, OTG_KIND_POINTS>;
using OctreeBoxF = OrthoTreeCoreGPU<BoundingBox3<float>, float, OTG_KIND_BOXES>;
// OctreeBoxs<IS_LOOSE_TREE> (core/ot_aliases.h:144-145): false = the regular box tree
template<bool IS_LOOSE_TREE>
using OctreeBoxs = OrthoTreeCoreGPU<BoundingBox3<double>, double, IS_LOOSE_TREE ? OTG_KIND_BOXES : OTG_KIND_BOXES_REGULAR>;
template<bool IS_LOOSE_TREE>
using OctreeBoxsF = OrthoTreeCoreGPU<BoundingBox3<float>, float, IS_LOOSE_TREE ? OTG_KIND_BOXES : OTG_KIND_BOXES_REGULAR>;

} // namespace OrthoTreeGPU
