// ref_harness.cpp — exposes the UNMODIFIED reference library (OrthoTree headers, compiled from
// their own location with -I) through the same C-ABI as otg_oracle_capi.cpp, so that the CPU
// restatement can be pinned against the reference itself and golden fixtures can be generated.
//
// TEST INFRASTRUCTURE ONLY. Built by oracle/Makefile into oracle/_ref/ (git-ignored), and only
// where the reference sources are present. Results are canonicalised exactly like the restatement's.
#include "orthotree/octree.h"
#include "orthotree/serialization.h"
#include "orthotree/serialization/binary_archive.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <span>
#include <sstream>
#include <string>
#include <vector>

using namespace OrthoTree;

namespace
{
template<typename T>
using PointTree = OrthoTreePointND<3, T>;
template<typename T>
using LooseBoxTree = OrthoTreeBoxND<3, true, T>;
template<typename T>
using BoxTree = OrthoTreeBoxND<3, false, T>;
template<typename T>
using StaticPointTree = StaticOrthoTreePointND<3, T>;
template<typename T>
using StaticLooseBoxTree = StaticOrthoTreeBoxND<3, true, T>;
template<typename T>
using StaticBoxTree = StaticOrthoTreeBoxND<3, false, T>;

struct Result
{
  std::vector<uint64_t> offsets{ 0 };
  std::vector<uint32_t> ids;
  std::vector<double> dist;
};

struct AnyRef
{
  int scalar = 0; // 0 double, 1 float
  int kind = 0;   // 0 points, 1 loose boxes, 2 boxes
  uint32_t D = 0;
  std::vector<double> ed;
  std::vector<float> ef;
  std::unique_ptr<PointTree<double>> pd;
  std::unique_ptr<LooseBoxTree<double>> lbd;
  std::unique_ptr<BoxTree<double>> bd;
  std::unique_ptr<PointTree<float>> pf;
  std::unique_ptr<LooseBoxTree<float>> lbf;
  std::unique_ptr<BoxTree<float>> bf;
  std::vector<uint64_t> locKeys;
  // the Create arguments, for the static tree of the same entities
  uint32_t maxDepthArg = 0;
  uint64_t maxElem = 16;
  bool hasBox = false;
  std::vector<double> boxd;
  std::vector<float> boxf;
};

template<typename T>
std::span<const PointND<3, T>> pts_span(const std::vector<T>& v)
{
  return { reinterpret_cast<const PointND<3, T>*>(v.data()), v.size() / 3 };
}
template<typename T>
std::span<const BoundingBoxND<3, T>> box_span(const std::vector<T>& v)
{
  return { reinterpret_cast<const BoundingBoxND<3, T>*>(v.data()), v.size() / 6 };
}

// StaticLinearOrthoTreeCore's arrays (ORTHOTREE__PUBLIC_LINEARDATA_INTERFACE), widened to 32 bits;
// `equal`: a loaded archive's tree IsEqualTo the reference's own tree of the same entities
struct StaticOut
{
  std::vector<uint32_t> childBegins, segments, entityStorage;
  std::vector<uint8_t> depth;
  std::vector<double> geometry;
  uint64_t geomPerNode = 3;
  int equal = 0;
};

template<typename StaticTree, typename T>
void static_args(const AnyRef* a, const std::vector<T>& box, std::optional<typename StaticTree::TBox>& ob, std::optional<depth_t>& od)
{
  if (a->hasBox)
    ob = *reinterpret_cast<const typename StaticTree::TBox*>(box.data());
  if (a->maxDepthArg)
    od = a->maxDepthArg;
}

template<typename StaticTree>
StaticOut* static_arrays(StaticTree const& t, bool isBox)
{
  auto* o = new StaticOut();
  std::visit(
    [&](auto const& nodes) {
      for (auto v : nodes.nodeChildSegmentBegins)
        o->childBegins.push_back(uint32_t(v));
      for (auto const& sg : nodes.nodeEntitySegment)
      {
        o->segments.push_back(uint32_t(sg.begin));
        o->segments.push_back(uint32_t(sg.length));
      }
    },
    t.GetNodes());
  o->depth.assign(t.GetNodeDepthIDs().begin(), t.GetNodeDepthIDs().end());
  o->entityStorage.assign(t.GetEntityStorage().begin(), t.GetEntityStorage().end());
  o->geomPerNode = isBox ? 6 : 3;
  for (auto const& g : t.GetNodeGeometries())
  {
    if constexpr (requires { g.minPoint; })
    {
      for (int d = 0; d < 3; ++d)
        o->geometry.push_back(double(g.minPoint[d]));
      for (int d = 0; d < 3; ++d)
        o->geometry.push_back(double(g.size[d]));
    }
    else
      for (int d = 0; d < 3; ++d)
        o->geometry.push_back(double(g[d]));
  }
  return o;
}

template<typename StaticTree, typename T, typename Span>
StaticOut* static_dump(Span ents, const AnyRef* a, const std::vector<T>& box, bool isBox)
{
  std::optional<typename StaticTree::TBox> ob;
  std::optional<depth_t> od;
  static_args<StaticTree>(a, box, ob, od);
  StaticTree t(PAR_EXEC, ents, od, ob, a->maxElem);
  return static_arrays(t, isBox);
}

// The reference's binary archive (serialization/binary_archive.h) of its static tree of the same
// entities: the core (`ar & tree`) or the Managed form with the entities.
template<typename StaticTree, typename T, typename Span>
std::string static_archive(Span ents, const AnyRef* a, const std::vector<T>& box, bool managed)
{
  std::optional<typename StaticTree::TBox> ob;
  std::optional<depth_t> od;
  static_args<StaticTree>(a, box, ob, od);
  std::stringstream ss(std::ios::in | std::ios::out | std::ios::binary);
  BinaryOutputArchive ar(ss);
  if (managed)
  {
    OrthoTreeManaged<StaticTree> m(ents, od, ob, a->maxElem, PAR_EXEC);
    ar & m;
  }
  else
  {
    StaticTree t(PAR_EXEC, ents, od, ob, a->maxElem);
    ar & t;
  }
  return ss.str();
}

// Loads archive bytes with the reference's BinaryInputArchive into its static tree type (null when
// the stream runs short or bytes are left over) and compares the loaded tree with the reference's
// own tree of the same entities: IsEqualTo both ways and, for the Managed form, equal entities.
template<typename StaticTree, typename T, typename Span>
StaticOut* static_load(Span ents, const AnyRef* a, const std::vector<T>& box, const std::string& bytes, bool managed, bool isBox)
{
  std::optional<typename StaticTree::TBox> ob;
  std::optional<depth_t> od;
  static_args<StaticTree>(a, box, ob, od);
  StaticTree own(PAR_EXEC, ents, od, ob, a->maxElem);
  std::stringstream ss(bytes, std::ios::in | std::ios::out | std::ios::binary);
  BinaryInputArchive ar(ss);
  auto finish = [&](StaticTree const& core, bool entitiesEqual) -> StaticOut* {
    if (!ss || ss.peek() != std::char_traits<char>::eof())
      return nullptr;
    auto* o = static_arrays(core, isBox);
    // IsEqualTo reads the root even when there is no node (empty trees): compare counts there
    const bool empty = core.GetNodeCount() == 0 || own.GetNodeCount() == 0;
    const bool same = empty ? core.GetNodeCount() == own.GetNodeCount() : core.IsEqualTo(own) && own.IsEqualTo(core);
    o->equal = entitiesEqual && same ? 1 : 0;
    return o;
  };
  if (managed)
  {
    OrthoTreeManaged<StaticTree> m;
    ar & m;
    auto const& data = m.GetData();
    bool same = data.size() == ents.size() && std::memcmp(data.data(), ents.data(), ents.size_bytes()) == 0;
    return finish(m.GetCore(), same);
  }
  StaticTree t;
  ar & t;
  return finish(t, true);
}

template<typename F>
auto with_static(AnyRef* a, F&& f)
{
  if (a->scalar == 0)
  {
    if (a->kind == 0)
      return f.template operator()<StaticPointTree<double>>(pts_span(a->ed), a->boxd, false);
    if (a->kind == 1)
      return f.template operator()<StaticLooseBoxTree<double>>(box_span(a->ed), a->boxd, true);
    return f.template operator()<StaticBoxTree<double>>(box_span(a->ed), a->boxd, true);
  }
  if (a->kind == 0)
    return f.template operator()<StaticPointTree<float>>(pts_span(a->ef), a->boxf, false);
  if (a->kind == 1)
    return f.template operator()<StaticLooseBoxTree<float>>(box_span(a->ef), a->boxf, true);
  return f.template operator()<StaticBoxTree<float>>(box_span(a->ef), a->boxf, true);
}


template<typename T>
T tol_or_default(double tol)
{
  return tol < 0 ? std::numeric_limits<T>::epsilon() * T(100) : T(tol);
}

// Location keys through the reference's own space indexing (si_mortongrid.h:69-97).
template<typename Tree, typename Span>
std::vector<uint64_t> location_keys(Span ents, const typename Tree::TBox* boxIn, uint32_t D)
{
  using GA = typename Tree::GA;
  using IGM = detail::InternalGeometryModule<GA>;
  using EA = typename Tree::EA;
  using CONFIG = typename Tree::CONFIG;
  auto space = boxIn ? IGM::GetBoxAD(*boxIn) : IGM::template GetBoundingBoxAD<EA>(ents);
  detail::MortonGridSpaceIndexing<GA, CONFIG::ALLOW_OUT_OF_SPACE_INSERTION, CONFIG::LOOSE_FACTOR, CONFIG::MAX_ALLOWED_DEPTH_ID> si(D, space);
  std::vector<uint64_t> keys(ents.size());
  for (size_t i = 0; i < ents.size(); ++i)
  {
    auto loc = si.GetLocation(ents[i]);
    keys[i] = (uint64_t(loc.GetLocationID()) << 5) | uint64_t(loc.GetDepthID());
  }
  return keys;
}

template<typename Tree>
void export_nodes(Tree const& t, uint64_t* keys, double* minp, double* size, uint64_t* eoff, uint32_t* eids)
{
  std::vector<uint64_t> ks;
  for (auto const& kv : t.GetNodes())
    ks.push_back(uint64_t(kv.first));
  std::sort(ks.begin(), ks.end());
  uint64_t off = 0;
  for (size_t i = 0; i < ks.size(); ++i)
  {
    auto nv = t.GetNodeValue(ks[i]);
    keys[i] = ks[i];
    auto const& mn = t.GetNodeMinPoint(nv);
    auto const& sz = t.GetNodeSize(nv);
    for (int d = 0; d < 3; ++d)
    {
      minp[3 * i + d] = double(mn[d]);
      size[3 * i + d] = double(sz[d]);
    }
    eoff[i] = off;
    std::vector<uint32_t> ids(t.GetNodeEntities(nv).begin(), t.GetNodeEntities(nv).end());
    std::sort(ids.begin(), ids.end());
    for (auto id : ids)
      eids[off++] = id;
  }
  eoff[ks.size()] = off;
}

// the key of every node's parent (the node whose child links hold it; 0 for the root and for nodes
// no link holds), nodes in ascending key order
template<typename Tree>
void export_parents(Tree const& t, uint64_t* parents)
{
  std::vector<uint64_t> ks;
  for (auto const& kv : t.GetNodes())
    ks.push_back(uint64_t(kv.first));
  std::sort(ks.begin(), ks.end());
  std::fill(parents, parents + ks.size(), 0);
  for (uint64_t k : ks)
    for (auto c : t.GetNodeChildren(t.GetNodeValue(k)))
    {
      const auto it = std::lower_bound(ks.begin(), ks.end(), uint64_t(c));
      if (it != ks.end() && *it == uint64_t(c))
        parents[it - ks.begin()] = k;
    }
}

template<typename F>
Result* run_queries(uint64_t nq, F&& one)
{
  auto* r = new Result();
  for (uint64_t q = 0; q < nq; ++q)
  {
    one(q, *r);
    r->offsets.push_back(r->ids.size());
  }
  return r;
}

template<typename T, typename Tree, typename Span>
Result* range_impl(Tree const& t, Span ents, const T* ranges, uint64_t nq, int mode, double tol)
{
  return run_queries(nq, [&](uint64_t q, Result& r) {
    auto const& b = *reinterpret_cast<const BoundingBoxND<3, T>*>(ranges + 6 * q);
    auto v = t.RangeSearch(b, ents, mode == 1 ? RangeSearchMode::Overlap : RangeSearchMode::Inside, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T, typename Tree, typename Span>
Result* pick_impl(Tree const& t, Span ents, const T* pts, uint64_t nq, double tol)
{
  return run_queries(nq, [&](uint64_t q, Result& r) {
    auto const& p = *reinterpret_cast<const PointND<3, T>*>(pts + 3 * q);
    auto v = t.PickSearch(p, ents, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T, typename Tree, typename Span>
Result* frustum_impl(Tree const& t, Span ents, const T* planes, uint64_t np, uint64_t nq, double tol)
{
  return run_queries(nq, [&](uint64_t q, Result& r) {
    std::vector<PlaneND<3, T>> pl(np);
    for (uint64_t i = 0; i < np; ++i)
    {
      const T* s = planes + 4 * (np * q + i);
      pl[i].OrigoDistance = s[0];
      pl[i].Normal = { s[1], s[2], s[3] };
    }
    auto v = t.FrustumCulling(std::span<const PlaneND<3, T>>(pl), ents, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T, typename Tree, typename Span>
Result* plane_impl(Tree const& t, Span ents, const T* planes, uint64_t nq, double tol, int positive)
{
  return run_queries(nq, [&](uint64_t q, Result& r) {
    const T* s = planes + 4 * q;
    PlaneND<3, T> pl;
    pl.OrigoDistance = s[0];
    pl.Normal = { s[1], s[2], s[3] };
    auto v = positive ? t.PlanePositiveSegmentation(pl, ents, tol_or_default<T>(tol)) : t.PlaneSearch(pl, ents, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
// one condition of a combined query, laid out as otg_condition in include/octree_gb300.h
struct CondC
{
  int32_t kind;
  uint32_t first;
  uint32_t count;
  uint32_t pad;
  double tol;
};
template<typename T, typename Tree, typename Span>
Result* query_impl(Tree const& t, Span ents, const CondC* conds, const uint64_t* off, uint64_t nq, const T* planes, const unsigned char* cross,
                   const T* boxes, int orOp, double tol)
{
  using Plane = PlaneND<3, T>;
  auto plane = [&](uint32_t j) {
    Plane p;
    p.OrigoDistance = planes[4 * j];
    p.Normal = { planes[4 * j + 1], planes[4 * j + 2], planes[4 * j + 3] };
    return p;
  };
  return run_queries(nq, [&](uint64_t q, Result& r) {
    std::vector<typename Tree::QueryCondition> c;
    for (uint64_t i = off[q]; i < off[q + 1]; ++i)
    {
      const CondC& k = conds[i];
      if (k.kind == 0)
      {
        std::vector<std::pair<Plane, bool>> ps;
        for (uint32_t j = k.first; j < k.first + k.count; ++j)
          ps.emplace_back(plane(j), cross[j] != 0);
        c.push_back(Tree::ByInFrustum(std::move(ps)));
      }
      else if (k.kind == 3)
        c.push_back(Tree::ByIntersecting(plane(k.first), k.tol < 0 ? tol_or_default<T>(-1.0) : T(k.tol)));
      else
      {
        const auto& b = *reinterpret_cast<const typename Tree::TBox*>(boxes + 6 * uint64_t(k.first));
        c.push_back(k.kind == 1 ? Tree::ByWithin(b) : Tree::ByOverlaps(b));
      }
    }
    auto v = orOp ? t.template Query<LogicalOperator::Or>(c, ents, tol_or_default<T>(tol))
                  : t.template Query<LogicalOperator::And>(c, ents, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T, bool IS_BOX, typename Tree, typename Span>
Result* knn_impl(Tree const& t, Span ents, const T* pts, uint64_t nq, const uint32_t* k, double maxDist, double tol)
{
  using GA = GeneralGeometryAdapterND<3, T>;
  T md = maxDist < 0 ? std::numeric_limits<T>::max() : T(maxDist);
  T tl = tol_or_default<T>(tol);
  return run_queries(nq, [&](uint64_t q, Result& r) {
    auto const& p = *reinterpret_cast<const PointND<3, T>*>(pts + 3 * q);
    auto v = t.template GetNearestNeighbors<true>(p, k[q], md, ents, tl);
    std::vector<std::pair<T, uint32_t>> dv;
    for (auto id : v)
    {
      T dist;
      if constexpr (IS_BOX)
        dist = GA::MinMaxDistance(p, ents[id], tl).min;
      else
        dist = GA::Distance(p, ents[id]);
      dv.emplace_back(dist, id);
    }
    std::sort(dv.begin(), dv.end());
    for (auto& e : dv)
    {
      r.ids.push_back(e.second);
      r.dist.push_back(double(e.first));
    }
  });
}
template<typename T, typename Tree, typename Span>
Result* ray_impl(Tree const& t, Span ents, const T* rays, uint64_t nq, double tol, double tolInc, double maxDist, bool first)
{
  using GA = GeneralGeometryAdapterND<3, T>;
  using IGM = detail::InternalGeometryModule<GA>;
  T md = maxDist < 0 ? std::numeric_limits<T>::max() : T(maxDist);
  T tl = tol_or_default<T>(tol);
  return run_queries(nq, [&](uint64_t q, Result& r) {
    auto const& o = *reinterpret_cast<const PointND<3, T>*>(rays + 6 * q);
    auto const& d = *reinterpret_cast<const PointND<3, T>*>(rays + 6 * q + 3);
    auto v = first ? t.RayIntersectedFirst(o, d, ents, tl, T(tolInc), md) : t.RayIntersectedAll(o, d, ents, tl, T(tolInc), md);
    auto rt = IGM::RayHitTester::Make(o, d, tl, T(tolInc));
    std::vector<std::pair<T, uint32_t>> dv;
    for (auto id : v)
    {
      auto h = rt->Hit(ents[id]);
      dv.emplace_back(h ? h->enterDistance : T(-1), id);
    }
    std::sort(dv.begin(), dv.end());
    for (auto& e : dv)
    {
      r.ids.push_back(e.second);
      r.dist.push_back(double(e.first));
    }
  });
}
Result* pairs_result(std::vector<std::pair<uint32_t, uint32_t>> p, bool canonical)
{
  if (canonical)
    for (auto& e : p)
      if (e.first > e.second)
        std::swap(e.first, e.second);
  std::sort(p.begin(), p.end());
  auto* r = new Result();
  for (auto& e : p)
  {
    r->ids.push_back(e.first);
    r->ids.push_back(e.second);
  }
  r->offsets.push_back(r->ids.size());
  return r;
}

// dispatch helper: calls f(tree, span, scalarTag)
template<typename F>
auto with_tree(AnyRef* a, F&& f)
{
  if (a->scalar == 0)
  {
    if (a->kind == 0)
      return f(*a->pd, pts_span(a->ed), double{}, std::false_type{});
    if (a->kind == 1)
      return f(*a->lbd, box_span(a->ed), double{}, std::true_type{});
    return f(*a->bd, box_span(a->ed), double{}, std::true_type{});
  }
  if (a->kind == 0)
    return f(*a->pf, pts_span(a->ef), float{}, std::false_type{});
  if (a->kind == 1)
    return f(*a->lbf, box_span(a->ef), float{}, std::true_type{});
  return f(*a->bf, box_span(a->ef), float{}, std::true_type{});
}

template<typename Tree, typename T, typename Span>
std::unique_ptr<Tree> make_tree(Span ents, uint32_t maxDepth, const T* box, uint64_t maxElem, AnyRef* a)
{
  std::optional<typename Tree::TBox> ob;
  if (box)
    ob = *reinterpret_cast<const typename Tree::TBox*>(box);
  std::optional<depth_t> od;
  if (maxDepth)
    od = maxDepth;
  auto t = std::make_unique<Tree>(PAR_EXEC, ents, od, ob, maxElem);
  a->D = t->GetMaxDepthID();
  a->locKeys = location_keys<Tree>(ents, box ? &*ob : nullptr, a->D);
  return t;
}
} // namespace

extern "C"
{
  void* oro_create(int scalar, int kind, const void* ent, uint64_t n, uint32_t maxDepth, const void* box, uint64_t maxElem)
  {
    auto* a = new AnyRef();
    a->scalar = scalar;
    a->kind = kind;
    a->maxDepthArg = maxDepth;
    a->maxElem = maxElem;
    a->hasBox = box != nullptr;
    if (box && scalar == 0)
      a->boxd.assign((const double*)box, (const double*)box + 6);
    if (box && scalar == 1)
      a->boxf.assign((const float*)box, (const float*)box + 6);
    size_t w = kind == 0 ? 3 : 6;
    if (scalar == 0)
    {
      a->ed.assign((const double*)ent, (const double*)ent + n * w);
      auto* b = (const double*)box;
      if (kind == 0)
        a->pd = make_tree<PointTree<double>>(pts_span(a->ed), maxDepth, b, maxElem, a);
      else if (kind == 1)
        a->lbd = make_tree<LooseBoxTree<double>>(box_span(a->ed), maxDepth, b, maxElem, a);
      else
        a->bd = make_tree<BoxTree<double>>(box_span(a->ed), maxDepth, b, maxElem, a);
    }
    else
    {
      a->ef.assign((const float*)ent, (const float*)ent + n * w);
      auto* b = (const float*)box;
      if (kind == 0)
        a->pf = make_tree<PointTree<float>>(pts_span(a->ef), maxDepth, b, maxElem, a);
      else if (kind == 1)
        a->lbf = make_tree<LooseBoxTree<float>>(box_span(a->ef), maxDepth, b, maxElem, a);
      else
        a->bf = make_tree<BoxTree<float>>(box_span(a->ef), maxDepth, b, maxElem, a);
    }
    return a;
  }
  void oro_destroy(void* h) { delete (AnyRef*)h; }
  uint32_t oro_max_depth(void* h) { return ((AnyRef*)h)->D; }
  uint64_t oro_node_count(void* h)
  {
    return with_tree((AnyRef*)h, [](auto& t, auto, auto, auto) { return uint64_t(t.GetNodeCount()); });
  }
  // The reference's static tree of the same entities (PAR_EXEC Create), or null for a point tree
  // holding points outside its space: the reference's static Build does not end on those when the
  // group of child 0 holds more than maxElem entities, so it is not called for them.
  void* oro_static(void* h)
  {
    auto* a = (AnyRef*)h;
    if (a->kind == 0)
      for (auto k : a->locKeys)
        if ((k & 31u) != a->D)
          return nullptr;
    if (a->scalar == 0)
    {
      if (a->kind == 0)
        return static_dump<StaticPointTree<double>>(pts_span(a->ed), a, a->boxd, false);
      if (a->kind == 1)
        return static_dump<StaticLooseBoxTree<double>>(box_span(a->ed), a, a->boxd, true);
      return static_dump<StaticBoxTree<double>>(box_span(a->ed), a, a->boxd, true);
    }
    if (a->kind == 0)
      return static_dump<StaticPointTree<float>>(pts_span(a->ef), a, a->boxf, false);
    if (a->kind == 1)
      return static_dump<StaticLooseBoxTree<float>>(box_span(a->ef), a, a->boxf, true);
    return static_dump<StaticBoxTree<float>>(box_span(a->ef), a, a->boxf, true);
  }
  void oro_static_sizes(void* s, uint64_t* sizes4)
  {
    auto* o = (StaticOut*)s;
    sizes4[0] = o->depth.size();
    sizes4[1] = o->childBegins.size();
    sizes4[2] = o->entityStorage.size();
    sizes4[3] = o->geomPerNode;
  }
  void oro_static_copy(void* s, uint32_t* childBegins, uint32_t* segments, uint8_t* depth, uint32_t* entityStorage, double* geometry)
  {
    auto* o = (StaticOut*)s;
    std::memcpy(childBegins, o->childBegins.data(), o->childBegins.size() * sizeof(uint32_t));
    std::memcpy(segments, o->segments.data(), o->segments.size() * sizeof(uint32_t));
    std::memcpy(depth, o->depth.data(), o->depth.size());
    std::memcpy(entityStorage, o->entityStorage.data(), o->entityStorage.size() * sizeof(uint32_t));
    std::memcpy(geometry, o->geometry.data(), o->geometry.size() * sizeof(double));
  }
  void oro_static_free(void* s) { delete (StaticOut*)s; }
  int oro_static_equal(void* s) { return ((StaticOut*)s)->equal; }

  // The reference's archive of its static tree (managed: with the entities); returns its size and
  // copies it when `cap` allows. Not for point trees with points outside their space (see oro_static).
  uint64_t oro_static_archive(void* h, int managed, uint8_t* buf, uint64_t cap)
  {
    auto* a = (AnyRef*)h;
    std::string bytes = with_static(a, [&]<typename ST>(auto ents, auto const& box, bool) { return static_archive<ST>(ents, a, box, managed != 0); });
    if (buf && cap >= bytes.size())
      std::memcpy(buf, bytes.data(), bytes.size());
    return bytes.size();
  }

  // The reference's own dynamicTree.IsEqualTo(staticTree) (core/ot_query.h:2149-2266) for its
  // dynamic tree and the static tree of the same entities; -1 where the static tree is not built
  // (point trees with points outside their space, see oro_static)
  int oro_dynamic_equals_static(void* h)
  {
    auto* a = (AnyRef*)h;
    if (a->kind == 0)
      for (auto k : a->locKeys)
        if ((k & 31u) != a->D)
          return -1;
    return with_static(a, [&]<typename ST>(auto ents, auto const& box, bool) -> int {
      std::optional<typename ST::TBox> ob;
      std::optional<depth_t> od;
      static_args<ST>(a, box, ob, od);
      ST st(PAR_EXEC, ents, od, ob, a->maxElem);
      return with_tree(a, [&](auto& dyn, auto, auto, auto) -> int {
        if constexpr (std::is_same_v<typename std::decay_t<decltype(dyn)>::GA, typename ST::GA>)
        {
          if (dyn.GetNodeCount() == 0 || st.GetNodeCount() == 0)
            return dyn.GetNodeCount() == st.GetNodeCount() ? 1 : 0;
          return dyn.IsEqualTo(st) ? 1 : 0;
        }
        else
          return -1;
      });
    });
  }

  // Archive bytes loaded by the reference (see static_load); null when they do not load.
  void* oro_static_load(void* h, const uint8_t* buf, uint64_t size, int managed)
  {
    auto* a = (AnyRef*)h;
    std::string bytes(reinterpret_cast<const char*>(buf), size);
    return with_static(a, [&]<typename ST>(auto ents, auto const& box, bool isBox) -> StaticOut* {
      return static_load<ST>(ents, a, box, bytes, managed != 0, isBox);
    });
  }

  void oro_location_keys(void* h, uint64_t* out)
  {
    auto* a = (AnyRef*)h;
    std::memcpy(out, a->locKeys.data(), a->locKeys.size() * sizeof(uint64_t));
  }
  void oro_export_nodes(void* h, uint64_t* keys, double* minp, double* size, uint64_t* eoff, uint32_t* eids, uint64_t* subtree)
  {
    (void)subtree;
    with_tree((AnyRef*)h, [&](auto& t, auto, auto, auto) {
      export_nodes(t, keys, minp, size, eoff, eids);
      return 0;
    });
  }
  void oro_node_parents(void* h, uint64_t* parents)
  {
    with_tree((AnyRef*)h, [&](auto& t, auto, auto, auto) {
      export_parents(t, parents);
      return 0;
    });
  }
  void* oro_range(void* h, const void* ranges, uint64_t nq, int mode, double tol)
  {
    return with_tree((AnyRef*)h, [&](auto& t, auto ents, auto s, auto) -> Result* {
      using T = decltype(s);
      return range_impl<T>(t, ents, (const T*)ranges, nq, mode, tol);
    });
  }
  void* oro_pick(void* h, const void* pts, uint64_t nq, double tol)
  {
    return with_tree((AnyRef*)h, [&](auto& t, auto ents, auto s, auto) -> Result* {
      using T = decltype(s);
      return pick_impl<T>(t, ents, (const T*)pts, nq, tol);
    });
  }
  void* oro_plane(void* h, const void* planes, uint64_t nq, double tol, int positive)
  {
    return with_tree((AnyRef*)h, [&](auto& t, auto ents, auto s, auto) -> Result* {
      using T = decltype(s);
      return plane_impl<T>(t, ents, (const T*)planes, nq, tol, positive);
    });
  }
  void* oro_query(void* h, const void* conds, const uint64_t* off, uint64_t nq, const void* planes, const unsigned char* cross, const void* boxes,
                  int or_op, double tol)
  {
    return with_tree((AnyRef*)h, [&](auto& t, auto ents, auto s, auto) -> Result* {
      using T = decltype(s);
      return query_impl<T>(t, ents, (const CondC*)conds, off, nq, (const T*)planes, cross, (const T*)boxes, or_op, tol);
    });
  }
  void* oro_frustum(void* h, const void* planes, uint64_t np, uint64_t nq, double tol)
  {
    return with_tree((AnyRef*)h, [&](auto& t, auto ents, auto s, auto) -> Result* {
      using T = decltype(s);
      return frustum_impl<T>(t, ents, (const T*)planes, np, nq, tol);
    });
  }
  void* oro_knn(void* h, const void* pts, uint64_t nq, const uint32_t* k, double maxDist, double tol)
  {
    return with_tree((AnyRef*)h, [&](auto& t, auto ents, auto s, auto isBox) -> Result* {
      using T = decltype(s);
      return knn_impl<T, decltype(isBox)::value>(t, ents, (const T*)pts, nq, k, maxDist, tol);
    });
  }
  void* oro_ray(void* h, const void* rays, uint64_t nq, double tol, double tolInc, double maxDist, int first)
  {
    return with_tree((AnyRef*)h, [&](auto& t, auto ents, auto s, auto) -> Result* {
      using T = decltype(s);
      return ray_impl<T>(t, ents, (const T*)rays, nq, tol, tolInc, maxDist, first != 0);
    });
  }
  void* oro_collide_self(void* h, double tol)
  {
    auto* a = (AnyRef*)h;
    if (a->kind == 0)
      return pairs_result({}, true);
    return with_tree(a, [&](auto& t, auto ents, auto s, auto isBox) -> Result* {
      using T = decltype(s);
      if constexpr (decltype(isBox)::value)
        return pairs_result(t.CollisionDetection(ents, tol_or_default<T>(tol), SEQ_EXEC), true);
      else
        return pairs_result({}, true);
    });
  }
  // Same as oro_collide_self but through the parallel (task-split) path of the reference.
  void* oro_collide_self_par(void* h, double tol)
  {
    auto* a = (AnyRef*)h;
    return with_tree(a, [&](auto& t, auto ents, auto s, auto isBox) -> Result* {
      using T = decltype(s);
      if constexpr (decltype(isBox)::value)
        return pairs_result(t.CollisionDetection(ents, tol_or_default<T>(tol), PAR_EXEC), true);
      else
        return pairs_result({}, true);
    });
  }
  void* oro_collide_pair(void* h1, void* h2, double tol)
  {
    auto* a = (AnyRef*)h1;
    auto* b = (AnyRef*)h2;
    if (a->scalar == 0 && a->kind == 1)
      return pairs_result(LooseBoxTree<double>::CollisionDetection(*a->lbd, box_span(a->ed), *b->lbd, box_span(b->ed), tol_or_default<double>(tol)), false);
    if (a->scalar == 1 && a->kind == 1)
      return pairs_result(LooseBoxTree<float>::CollisionDetection(*a->lbf, box_span(a->ef), *b->lbf, box_span(b->ef), tol_or_default<float>(tol)), false);
    if (a->scalar == 0 && a->kind == 2)
      return pairs_result(BoxTree<double>::CollisionDetection(*a->bd, box_span(a->ed), *b->bd, box_span(b->ed), tol_or_default<double>(tol)), false);
    if (a->scalar == 1 && a->kind == 2)
      return pairs_result(BoxTree<float>::CollisionDetection(*a->bf, box_span(a->ef), *b->bf, box_span(b->ef), tol_or_default<float>(tol)), false);
    return pairs_result({}, false);
  }
  uint64_t oro_res_nq(void* r) { return ((Result*)r)->offsets.size() - 1; }
  uint64_t oro_res_total(void* r) { return ((Result*)r)->ids.size(); }
  int oro_res_has_dist(void* r) { return ((Result*)r)->dist.empty() ? 0 : 1; }
  void oro_res_copy(void* rr, uint64_t* offsets, uint32_t* ids, double* dist)
  {
    auto* r = (Result*)rr;
    std::memcpy(offsets, r->offsets.data(), r->offsets.size() * sizeof(uint64_t));
    std::memcpy(ids, r->ids.data(), r->ids.size() * sizeof(uint32_t));
    if (dist && !r->dist.empty())
      std::memcpy(dist, r->dist.data(), r->dist.size() * sizeof(double));
  }
  void oro_res_free(void* r) { delete (Result*)r; }

  // Bulk Insert of n new points into a point tree (Insert(newEntities, existingEntities),
  // core/ot_dynamic_hash_core.h:1012-1333); the new entities get ids N .. N + n - 1 and join the span
  // that later queries pass. Returns the reference's result (all inserted).
  int oro_insert(void* h, const void* ent, uint64_t n)
  {
    auto* a = (AnyRef*)h;
    if (a->kind != 0)
      return 0;
    if (a->scalar == 0)
    {
      std::vector<double> add((const double*)ent, (const double*)ent + 3 * n);
      const bool ok = a->pd->Insert(pts_span(add), pts_span(a->ed));
      a->ed.insert(a->ed.end(), add.begin(), add.end());
      return ok ? 1 : 0;
    }
    std::vector<float> add((const float*)ent, (const float*)ent + 3 * n);
    const bool ok = a->pf->Insert(pts_span(add), pts_span(a->ef));
    a->ef.insert(a->ef.end(), add.begin(), add.end());
    return ok ? 1 : 0;
  }

  // Core form: the entity span that every later query passes (the tree is not rebuilt): the
  // reference's Core queries test the geometry of the span they are given against the nodes
  // Create built from the earlier one
  void oro_set_entities(void* h, const void* ent, uint64_t n)
  {
    auto* a = (AnyRef*)h;
    const uint64_t w = n * (a->kind == 0 ? 3 : 6);
    if (a->scalar == 0)
      a->ed.assign((const double*)ent, (const double*)ent + w);
    else
      a->ef.assign((const float*)ent, (const float*)ent + w);
  }

  // Timed reference Create (OctreePoint, PAR_EXEC) — used for the CPU baseline where the reference is built.
  double oro_time_create_points(const double* pts, uint64_t n, uint32_t maxDepth, uint64_t maxElem, int reps)
  {
    auto span = std::span<const Point3D>(reinterpret_cast<const Point3D*>(pts), n);
    auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < reps; ++r)
    {
      OctreePoint t(PAR_EXEC, span, depth_t(maxDepth), std::nullopt, maxElem);
      (void)t;
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
  }
}
