// otg_oracle_capi.cpp — C-ABI over the CPU restatement in otg_oracle.hpp.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/ (ctypes), __graft_entry__.smoke() and bench.py's
// CPU baseline. It is never linked into the GPU library.
//
// Results are returned canonicalised so that they can be compared with the GPU path:
//   range / pick / frustum : ids ascending
//   kNN                    : by (distance, id)          (reference returns by distance, ties unspecified)
//   ray all / ray first    : by (enter distance, id)    (RayIntersectedFirst returns farthest first)
//   collision pairs        : (min id, max id) ascending (reference pair orientation is not canonical)
#include "otg_oracle.hpp"

#include <chrono>
#include <cstring>
#include <memory>
#include <thread>

using namespace otg_oracle;

namespace
{
struct AnyTree
{
  int scalar = 0; // 0 double, 1 float
  std::unique_ptr<Tree<double>> d;
  std::unique_ptr<Tree<float>> f;
};

struct Result
{
  std::vector<uint64_t> offsets{ 0 };
  std::vector<uint32_t> ids;
  std::vector<double> dist;
};

// static layout flattened for the C-ABI: segments as {begin, length} pairs, geometry widened to double
struct StaticOut
{
  std::vector<uint32_t> childBegins, segments, entityStorage;
  std::vector<uint8_t> depth;
  std::vector<double> geometry;
  uint64_t geomPerNode = 3;
};

template<typename T>
bool fill_static(const Tree<T>& t, StaticOut& o)
{
  typename Tree<T>::StaticLayout s;
  if (!t.static_layout(s))
    return false;
  o.childBegins = s.childBegins;
  o.segments.resize(2 * s.segBegin.size());
  for (size_t i = 0; i < s.segBegin.size(); ++i)
  {
    o.segments[2 * i] = s.segBegin[i];
    o.segments[2 * i + 1] = s.segLength[i];
  }
  o.depth.assign(s.depth.begin(), s.depth.end());
  o.entityStorage = s.entityStorage;
  o.geometry.assign(s.geometry.begin(), s.geometry.end());
  o.geomPerNode = t.isBox ? 6 : 3;
  return true;
}

template<typename T>
T tol_or_default(double tol)
{
  return tol < 0 ? base_tolerance<T>() : T(tol);
}

template<typename T>
void sort_ids(std::vector<uint32_t>& v)
{
  std::sort(v.begin(), v.end());
}

template<typename T, typename F>
Result* run_queries(uint64_t nq, F&& one)
{
  auto* r = new Result();
  r->offsets.reserve(nq + 1);
  for (uint64_t q = 0; q < nq; ++q)
  {
    one(q, *r);
    r->offsets.push_back(r->ids.size());
  }
  return r;
}

template<typename T>
Result* range_impl(Tree<T>& t, const T* ranges, uint64_t nq, int mode, double tol)
{
  return run_queries<T>(nq, [&](uint64_t q, Result& r) {
    auto v = t.range_search(ranges + 6 * q, mode == 1 ? RangeMode::Overlap : RangeMode::Inside, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T>
Result* pick_impl(Tree<T>& t, const T* pts, uint64_t nq, double tol)
{
  return run_queries<T>(nq, [&](uint64_t q, Result& r) {
    auto v = t.pick_search(pts + 3 * q, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T>
Result* frustum_impl(Tree<T>& t, const T* planes, uint64_t np, uint64_t nq, double tol)
{
  return run_queries<T>(nq, [&](uint64_t q, Result& r) {
    auto v = t.frustum(planes + 4 * np * q, np, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T>
Result* plane_impl(Tree<T>& t, const T* planes, uint64_t nq, double tol, int positive)
{
  return run_queries<T>(nq, [&](uint64_t q, Result& r) {
    auto v = positive ? t.plane_positive(planes + 4 * q, tol_or_default<T>(tol)) : t.plane_search(planes + 4 * q, tol_or_default<T>(tol));
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
template<typename T>
Result* query_impl(Tree<T>& t, const CondC* conds, const uint64_t* off, uint64_t nq, const T* planes, const unsigned char* cross, const T* boxes,
                   int orOp, double tol)
{
  return run_queries<T>(nq, [&](uint64_t q, Result& r) {
    std::vector<typename Tree<T>::Cond> c;
    for (uint64_t i = off[q]; i < off[q + 1]; ++i)
      c.push_back({ conds[i].kind, conds[i].first, conds[i].count, conds[i].tol });
    auto v = t.query(c.data(), c.size(), planes, cross, boxes, orOp != 0, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end());
    r.ids.insert(r.ids.end(), v.begin(), v.end());
  });
}
template<typename T>
Result* knn_impl(Tree<T>& t, const T* pts, uint64_t nq, const uint32_t* k, double maxDist, double tol)
{
  T md = maxDist < 0 ? std::numeric_limits<T>::max() : T(maxDist);
  return run_queries<T>(nq, [&](uint64_t q, Result& r) {
    auto v = t.knn(pts + 3 * q, k[q], md, tol_or_default<T>(tol));
    std::sort(v.begin(), v.end(), [](auto& a, auto& b) { return a.distance < b.distance || (a.distance == b.distance && a.id < b.id); });
    for (auto& e : v)
    {
      r.ids.push_back(e.id);
      r.dist.push_back(double(e.distance));
    }
  });
}
template<typename T>
Result* ray_impl(Tree<T>& t, const T* rays, uint64_t nq, double tol, double tolInc, double maxDist, bool first)
{
  T md = maxDist < 0 ? std::numeric_limits<T>::max() : T(maxDist);
  return run_queries<T>(nq, [&](uint64_t q, Result& r) {
    const T* ray = rays + 6 * q;
    auto v = first ? t.ray_first(ray, ray + 3, tol_or_default<T>(tol), T(tolInc), md) : t.ray_all(ray, ray + 3, tol_or_default<T>(tol), T(tolInc), md);
    std::sort(v.begin(), v.end(), [](auto& a, auto& b) { return a.second < b.second || (a.second == b.second && a.first < b.first); });
    for (auto& e : v)
    {
      r.ids.push_back(e.first);
      r.dist.push_back(double(e.second));
    }
  });
}
Result* pairs_result(std::vector<std::pair<uint32_t, uint32_t>>& p)
{
  for (auto& e : p)
    if (e.first > e.second)
      std::swap(e.first, e.second);
  std::sort(p.begin(), p.end());
  auto* r = new Result();
  r->ids.reserve(p.size() * 2);
  for (auto& e : p)
  {
    r->ids.push_back(e.first);
    r->ids.push_back(e.second);
  }
  r->offsets.push_back(r->ids.size());
  return r;
}

template<typename T>
void export_nodes_impl(Tree<T>& t, uint64_t* keys, double* minp, double* size, uint64_t* eoff, uint32_t* eids, uint64_t* subtree)
{
  std::vector<uint64_t> ks;
  ks.reserve(t.nodes.size());
  for (auto& [k, n] : t.nodes)
    ks.push_back(k);
  std::sort(ks.begin(), ks.end());
  uint64_t off = 0;
  for (size_t i = 0; i < ks.size(); ++i)
  {
    auto& n = t.nodes.at(ks[i]);
    keys[i] = ks[i];
    const T* mn = t.node_min(n);
    const T* sz = t.node_size(n);
    for (int d = 0; d < 3; ++d)
    {
      minp[3 * i + d] = double(mn[d]);
      size[3 * i + d] = double(sz[d]);
    }
    if (subtree)
      subtree[i] = n.subtreeCount;
    eoff[i] = off;
    std::vector<uint32_t> ids(n.entities);
    std::sort(ids.begin(), ids.end());
    for (auto id : ids)
      eids[off++] = id;
  }
  eoff[ks.size()] = off;
}
// the key of every node's parent (0 for the root and for nodes no link holds), ascending key order
template<typename T>
void export_parents_impl(Tree<T>& t, uint64_t* parents)
{
  std::vector<uint64_t> ks;
  for (auto& [k, n] : t.nodes)
    ks.push_back(k);
  std::sort(ks.begin(), ks.end());
  std::fill(parents, parents + ks.size(), 0);
  for (uint64_t k : ks)
    for (uint64_t c : t.nodes.at(k).children)
    {
      const auto it = std::lower_bound(ks.begin(), ks.end(), c);
      if (it != ks.end() && *it == c)
        parents[it - ks.begin()] = k;
    }
}
} // namespace

extern "C"
{
  // kind: 0 points, 1 loose boxes (OctreeBox), 2 non-loose boxes. scalar: 0 double, 1 float.
  // box: 6 scalars (min xyz, max xyz) or NULL; maxDepth 0 = EstimateMaxDepth.
  // threads: workers of the location transform and the sort (the reference's ParExec steps)
  void* oro_create_threads(int scalar, int kind, const void* ent, uint64_t n, uint32_t maxDepth, const void* box, uint64_t maxElem, unsigned threads)
  {
    auto* a = new AnyTree();
    a->scalar = scalar;
    if (scalar == 0)
    {
      a->d = std::make_unique<Tree<double>>();
      a->d->threads = std::max(1u, threads);
      a->d->create((const double*)ent, n, maxDepth, (const double*)box, maxElem, kind != 0, kind == 1);
    }
    else
    {
      a->f = std::make_unique<Tree<float>>();
      a->f->threads = std::max(1u, threads);
      a->f->create((const float*)ent, n, maxDepth, (const float*)box, maxElem, kind != 0, kind == 1);
    }
    return a;
  }
  // Work counters of the reference's traversal (Tree::QueryWork): on = 1 clears them and starts
  // counting the tree's range and kNN queries (single-threaded calls only); oro_work reads them as
  // {node records, entity records, ids}.
  void oro_count_work(void* h, int on)
  {
    auto* a = (AnyTree*)h;
    if (a->scalar == 0)
    {
      a->d->countWork = on != 0;
      a->d->work = {};
    }
    else
    {
      a->f->countWork = on != 0;
      a->f->work = {};
    }
  }
  void oro_work(void* h, uint64_t* out3)
  {
    auto* a = (AnyTree*)h;
    auto put = [&](const auto& w) {
      out3[0] = w.nodes;
      out3[1] = w.entities;
      out3[2] = w.ids;
    };
    if (a->scalar == 0)
      put(a->d->work);
    else
      put(a->f->work);
  }
  void* oro_create(int scalar, int kind, const void* ent, uint64_t n, uint32_t maxDepth, const void* box, uint64_t maxElem)
  {
    return oro_create_threads(scalar, kind, ent, n, maxDepth, box, maxElem, 1);
  }
  void oro_destroy(void* h) { delete (AnyTree*)h; }
  // Bulk Insert of n new points (Tree::insert_points); 1 when they were inserted, 0 when refused
  int oro_insert(void* h, const void* ent, uint64_t n)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? int(a->d->insert_points((const double*)ent, n)) : int(a->f->insert_points((const float*)ent, n));
  }
  // Core form: `ent` (n entities, the Create layout) becomes the geometry the tree's queries test;
  // the nodes stay as Create built them (the reference's Core queries take the span per call)
  void oro_set_entities(void* h, const void* ent, uint64_t n)
  {
    auto* a = (AnyTree*)h;
    if (a->scalar == 0)
      a->d->geom.assign((const double*)ent, (const double*)ent + n * (a->d->isBox ? 6 : 3));
    else
      a->f->geom.assign((const float*)ent, (const float*)ent + n * (a->f->isBox ? 6 : 3));
  }
  uint32_t oro_max_depth(void* h)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? a->d->D : a->f->D;
  }
  uint64_t oro_node_count(void* h)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? a->d->nodes.size() : a->f->nodes.size();
  }
  // per-entity compact location key (loc << 5 | depth), input order
  // Static linear layout (Tree::static_layout): a handle, or null where the layout is undefined.
  // Sizes: {nodes, stored child segment begins, entities, scalars of geometry per node}.
  void* oro_static(void* h)
  {
    auto* a = (AnyTree*)h;
    auto* out = new StaticOut();
    bool ok = a->scalar == 0 ? fill_static(*a->d, *out) : fill_static(*a->f, *out);
    if (!ok)
    {
      delete out;
      return nullptr;
    }
    return out;
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

  void oro_location_keys(void* h, uint64_t* out)
  {
    auto* a = (AnyTree*)h;
    auto& v = a->scalar == 0 ? a->d->locationKeys : a->f->locationKeys;
    std::memcpy(out, v.data(), v.size() * sizeof(uint64_t));
  }
  // grid space: min[3], max[3], node size table (points) of depth 0..D+1 (3 per depth)
  void oro_space(void* h, double* minmax6)
  {
    auto* a = (AnyTree*)h;
    for (int d = 0; d < 3; ++d)
    {
      minmax6[d] = a->scalar == 0 ? a->d->spaceMin[d] : a->f->spaceMin[d];
      minmax6[3 + d] = a->scalar == 0 ? a->d->spaceMax[d] : a->f->spaceMax[d];
    }
  }
  // nodes sorted by key; own entities of node i are eids[eoff[i] : eoff[i+1]] (ascending)
  void oro_export_nodes(void* h, uint64_t* keys, double* minp, double* size, uint64_t* eoff, uint32_t* eids, uint64_t* subtree)
  {
    auto* a = (AnyTree*)h;
    if (a->scalar == 0)
      export_nodes_impl(*a->d, keys, minp, size, eoff, eids, subtree);
    else
      export_nodes_impl(*a->f, keys, minp, size, eoff, eids, subtree);
  }

  void oro_node_parents(void* h, uint64_t* parents)
  {
    auto* a = (AnyTree*)h;
    if (a->scalar == 0)
      export_parents_impl(*a->d, parents);
    else
      export_parents_impl(*a->f, parents);
  }
  void* oro_range(void* h, const void* ranges, uint64_t nq, int mode, double tol)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? range_impl(*a->d, (const double*)ranges, nq, mode, tol) : range_impl(*a->f, (const float*)ranges, nq, mode, tol);
  }
  void* oro_pick(void* h, const void* pts, uint64_t nq, double tol)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? pick_impl(*a->d, (const double*)pts, nq, tol) : pick_impl(*a->f, (const float*)pts, nq, tol);
  }
  // one plane per query; positive = 0: PlaneSearch, 1: PlanePositiveSegmentation
  void* oro_plane(void* h, const void* planes, uint64_t nq, double tol, int positive)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? plane_impl(*a->d, (const double*)planes, nq, tol, positive) : plane_impl(*a->f, (const float*)planes, nq, tol, positive);
  }
  // combined queries: query q holds conditions [off[q], off[q + 1]); or_op 0: And, 1: Or
  void* oro_query(void* h, const void* conds, const uint64_t* off, uint64_t nq, const void* planes, const unsigned char* cross, const void* boxes,
                  int or_op, double tol)
  {
    auto* a = (AnyTree*)h;
    const CondC* c = (const CondC*)conds;
    return a->scalar == 0 ? query_impl(*a->d, c, off, nq, (const double*)planes, cross, (const double*)boxes, or_op, tol)
                          : query_impl(*a->f, c, off, nq, (const float*)planes, cross, (const float*)boxes, or_op, tol);
  }
  void* oro_frustum(void* h, const void* planes, uint64_t np, uint64_t nq, double tol)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? frustum_impl(*a->d, (const double*)planes, np, nq, tol) : frustum_impl(*a->f, (const float*)planes, np, nq, tol);
  }
  // maxDist < 0: unbounded (numeric_limits<T>::max())
  void* oro_knn(void* h, const void* pts, uint64_t nq, const uint32_t* k, double maxDist, double tol)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? knn_impl(*a->d, (const double*)pts, nq, k, maxDist, tol) : knn_impl(*a->f, (const float*)pts, nq, k, maxDist, tol);
  }
  void* oro_ray(void* h, const void* rays, uint64_t nq, double tol, double tolInc, double maxDist, int first)
  {
    auto* a = (AnyTree*)h;
    return a->scalar == 0 ? ray_impl(*a->d, (const double*)rays, nq, tol, tolInc, maxDist, first != 0)
                          : ray_impl(*a->f, (const float*)rays, nq, tol, tolInc, maxDist, first != 0);
  }
  void* oro_collide_self(void* h, double tol)
  {
    auto* a = (AnyTree*)h;
    if (a->scalar == 0)
    {
      auto p = a->d->collide_self(tol_or_default<double>(tol));
      return pairs_result(p);
    }
    auto p = a->f->collide_self(tol_or_default<float>(tol));
    return pairs_result(p);
  }
  void* oro_collide_pair(void* h1, void* h2, double tol)
  {
    auto* a = (AnyTree*)h1;
    auto* b = (AnyTree*)h2;
    if (a->scalar == 0)
    {
      auto p = Tree<double>::collide_pair(*a->d, *b->d, tol_or_default<double>(tol));
      // two-tree pairs are (left id, right id): keep orientation, sort
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
    auto p = Tree<float>::collide_pair(*a->f, *b->f, tol_or_default<float>(tol));
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

  // Brute force O(N^2) references used by tests (adapters/general.h predicates only).
  void* oro_brute_collide(int scalar, const void* boxes, uint64_t n, double tol)
  {
    std::vector<std::pair<uint32_t, uint32_t>> p;
    if (scalar == 0)
    {
      auto* b = (const double*)boxes;
      double t = tol_or_default<double>(tol);
      for (uint64_t i = 0; i < n; ++i)
        for (uint64_t j = i + 1; j < n; ++j)
          if (Geo<double>::overlapped_strict(b + 6 * i, b + 6 * j, t))
            p.emplace_back(uint32_t(i), uint32_t(j));
    }
    else
    {
      auto* b = (const float*)boxes;
      float t = tol_or_default<float>(tol);
      for (uint64_t i = 0; i < n; ++i)
        for (uint64_t j = i + 1; j < n; ++j)
          if (Geo<float>::overlapped_strict(b + 6 * i, b + 6 * j, t))
            p.emplace_back(uint32_t(i), uint32_t(j));
    }
    return pairs_result(p);
  }

  // Timed CPU baseline helper: builds and destroys `reps` trees (points, double), returns seconds.
  // threads: workers of the location transform and the sort (the reference's ParExec steps)
  double oro_time_create_points_par(const double* pts, uint64_t n, uint32_t maxDepth, uint64_t maxElem, int reps, unsigned threads)
  {
    auto t0 = std::chrono::steady_clock::now();
    for (int r = 0; r < reps; ++r)
    {
      Tree<double> t;
      t.threads = std::max(1u, threads);
      t.create(pts, n, maxDepth, nullptr, maxElem, false, false);
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
  }
  double oro_time_create_points(const double* pts, uint64_t n, uint32_t maxDepth, uint64_t maxElem, int reps)
  {
    return oro_time_create_points_par(pts, n, maxDepth, maxElem, reps, 1);
  }
}
