// Drop-in test of include/orthotree_gpu.hpp: builds point and box trees through the C++ types and
// compares every query with the CPU oracle (oracle/otg_oracle_capi.cpp, linked as test
// infrastructure). Without a CUDA device it checks that the types fail loudly instead.
//   exit 0 and "OK" on success; any mismatch prints the query and exits 1.
#include "orthotree_gpu.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <unordered_set>
#include <vector>

extern "C"
{
  void* oro_create(int scalar, int kind, const void* ent, uint64_t n, uint32_t maxDepth, const void* box, uint64_t maxElem);
  void oro_destroy(void* h);
  void* oro_range(void* h, const void* ranges, uint64_t nq, int mode, double tol);
  void* oro_pick(void* h, const void* pts, uint64_t nq, double tol);
  void* oro_knn(void* h, const void* pts, uint64_t nq, const uint32_t* k, double maxDist, double tol);
  void* oro_ray(void* h, const void* rays, uint64_t nq, double tol, double tolInc, double maxDist, int first);
  void* oro_frustum(void* h, const void* planes, uint64_t np, uint64_t nq, double tol);
  void* oro_plane(void* h, const void* planes, uint64_t nq, double tol, int positive);
  void* oro_query(void* h, const void* conds, const uint64_t* off, uint64_t nq, const void* planes, const unsigned char* cross, const void* boxes,
                  int or_op, double tol);
  void* oro_collide_self(void* h, double tol);
  void* oro_collide_pair(void* h1, void* h2, double tol);
  void oro_set_entities(void* h, const void* ent, uint64_t n);
  int oro_insert(void* h, const void* ent, uint64_t n);
  uint64_t oro_res_nq(void* r);
  uint64_t oro_res_total(void* r);
  void oro_res_copy(void* r, uint64_t* offsets, uint32_t* ids, double* dist);
  void oro_res_free(void* r);
  void* oro_static(void* h);
  void oro_static_sizes(void* s, uint64_t* sizes4);
  void oro_static_copy(void* s, uint32_t* childBegins, uint32_t* segments, uint8_t* depth, uint32_t* entityStorage, double* geometry);
  void oro_static_free(void* s);
}

using namespace OrthoTreeGPU;

static int g_fail = 0;

static std::vector<uint32_t> oracle_ids(void* r, uint64_t q)
{
  std::vector<uint64_t> off(oro_res_nq(r) + 1);
  std::vector<uint32_t> ids(oro_res_total(r));
  std::vector<double> dist(ids.size());
  oro_res_copy(r, off.data(), ids.data(), dist.data());
  return { ids.begin() + off[q], ids.begin() + off[q + 1] };
}

static void expect(const std::vector<uint32_t>& got, void* oracleResult, uint64_t q, const char* what)
{
  auto want = oracle_ids(oracleResult, q);
  if (got != want)
  {
    std::printf("MISMATCH %s query %llu: %zu vs %zu ids\n", what, (unsigned long long)q, got.size(), want.size());
    ++g_fail;
  }
}

int main()
{
  if (otg_device_count() == 0)
  {
    try
    {
      std::vector<Point3D> pts(16, Point3D{ 0, 0, 0 });
      OctreePointM t(pts, 4);
      std::printf("no exception without a device\n");
      return 1;
    }
    catch (const Error& e)
    {
      if (e.status() != OTG_ERR_NO_DEVICE)
        return 1;
      std::printf("OK (no device: %s)\n", e.what());
      return 0;
    }
  }

  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(0.0, 100.0), E(0.05, 3.0);
  // ---- points
  std::vector<Point3D> pts(50000);
  for (auto& p : pts)
    p = { U(rng), U(rng), U(rng) };
  OctreePointM tp(pts, 8, std::nullopt, 20);
  void* op = oro_create(0, 0, pts.data(), pts.size(), 8, nullptr, 20);
  const int nq = 64;
  std::vector<BoundingBox3D> ranges(nq);
  std::vector<Point3D> qp(nq);
  std::vector<Ray3D> rays(nq);
  std::normal_distribution<double> N(0.0, 1.0);
  for (int i = 0; i < nq; ++i)
  {
    const Point3D c{ U(rng), U(rng), U(rng) };
    const double e = E(rng);
    ranges[i] = { { c[0] - e, c[1] - e, c[2] - e }, { c[0] + e, c[1] + e, c[2] + e } };
    qp[i] = { U(rng), U(rng), U(rng) };
    Point3D d{ N(rng), N(rng), N(rng) };
    const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    rays[i] = { qp[i], { d[0] / l, d[1] / l, d[2] / l } };
  }
  {
    void* r = oro_range(op, ranges.data(), nq, 0, -1.0);
    for (int i = 0; i < nq; ++i)
      expect(tp.RangeSearch(ranges[i]), r, i, "RangeSearch");
    oro_res_free(r);
    std::vector<uint32_t> k(nq, 9);
    r = oro_knn(op, qp.data(), nq, k.data(), -1.0, -1.0);
    for (int i = 0; i < nq; ++i)
      expect(tp.GetNearestNeighbors(qp[i], 9), r, i, "GetNearestNeighbors");
    oro_res_free(r);
    const Csr batch = tp.GetNearestNeighborsBatch(std::span<const Point3D>(qp), 9);
    r = oro_knn(op, qp.data(), nq, k.data(), -1.0, -1.0);
    for (int i = 0; i < nq; ++i)
      expect({ batch[i].begin(), batch[i].end() }, r, i, "GetNearestNeighborsBatch");
    oro_res_free(r);
  }
  // the static form: ExportStatic against the oracle's restatement, and an archive round trip
  {
    const auto sl = tp.ExportStatic();
    void* os = oro_static(op);
    uint64_t sz[4];
    oro_static_sizes(os, sz);
    std::vector<uint32_t> cb(sz[1]), seg(2 * sz[0]), es(sz[2]);
    std::vector<uint8_t> dep(sz[0]);
    std::vector<double> geo(sz[0] * sz[3]);
    oro_static_copy(os, cb.data(), seg.data(), dep.data(), es.data(), geo.data());
    oro_static_free(os);
    bool same = sl.nodeChildSegmentBegins == cb && sl.nodeDepthIDs == dep && sl.entityStorage == es && sl.nodeGeometry.size() == geo.size();
    for (std::size_t i = 0; same && i < sl.nodeEntitySegment.size(); ++i)
      same = sl.nodeEntitySegment[i].first == seg[2 * i] && sl.nodeEntitySegment[i].second == seg[2 * i + 1];
    for (std::size_t i = 0; same && i < geo.size(); ++i)
      same = sl.nodeGeometry[i] == geo[i];
    if (!same)
    {
      std::printf("MISMATCH ExportStatic\n");
      ++g_fail;
    }
    const auto archive = tp.SaveStatic();
    OctreePointM resumed;
    resumed.LoadStatic(archive);
    if (resumed.SaveStatic() != archive || resumed.RangeSearch(ranges[0]) != tp.RangeSearch(ranges[0]))
    {
      std::printf("MISMATCH SaveStatic / LoadStatic\n");
      ++g_fail;
    }
  }
  oro_destroy(op);

  // ---- boxes
  std::vector<BoundingBox3D> boxes(20000);
  for (auto& b : boxes)
  {
    const Point3D c{ U(rng), U(rng), U(rng) };
    const double e = E(rng) * 0.3;
    b = { { c[0] - e, c[1] - e, c[2] - e }, { c[0] + e, c[1] + e, c[2] + e } };
  }
  OctreeBoxM tb(boxes, 7, std::nullopt, 16);
  void* ob = oro_create(0, 1, boxes.data(), boxes.size(), 7, nullptr, 16);
  {
    void* r = oro_pick(ob, qp.data(), nq, -1.0);
    for (int i = 0; i < nq; ++i)
      expect(tb.PickSearch(qp[i]), r, i, "PickSearch");
    oro_res_free(r);
    r = oro_range(ob, ranges.data(), nq, 1, -1.0);
    for (int i = 0; i < nq; ++i)
      expect(tb.RangeSearch(ranges[i], RangeSearchMode::Overlap), r, i, "RangeSearch overlap");
    oro_res_free(r);
    r = oro_ray(ob, rays.data(), nq, -1.0, 0.0, -1.0, 0);
    for (int i = 0; i < nq; ++i)
      expect(tb.RayIntersectedAll(rays[i]), r, i, "RayIntersectedAll");
    oro_res_free(r);
    r = oro_ray(ob, rays.data(), nq, -1.0, 0.0, -1.0, 1);
    for (int i = 0; i < nq; ++i)
    {
      auto got = tb.RayIntersectedFirst(rays[i]);
      std::reverse(got.begin(), got.end()); // farthest first -> the oracle's (distance, id) order
      expect(got, r, i, "RayIntersectedFirst");
    }
    oro_res_free(r);
    std::vector<Plane3D> planes = { { 20.0, { 1, 0, 0 } }, { -80.0, { -1, 0, 0 } }, { 30.0, { 0, 1, 0 } },
                                    { -70.0, { 0, -1, 0 } }, { 10.0, { 0, 0, 1 } }, { -60.0, { 0, 0, -1 } } };
    r = oro_frustum(ob, planes.data(), planes.size(), 1, -1.0);
    expect(tb.FrustumCulling(planes), r, 0, "FrustumCulling");
    oro_res_free(r);
    const Plane3D cut{ 45.0, { 0.6, 0.8, 0.0 } };
    r = oro_plane(ob, &cut, 1, 0.5, 0);
    expect(tb.PlaneSearch(cut, 0.5), r, 0, "PlaneSearch");
    oro_res_free(r);
    r = oro_plane(ob, &cut, 1, -1.0, 1);
    expect(tb.PlanePositiveSegmentation(cut), r, 0, "PlanePositiveSegmentation");
    oro_res_free(r);
    // Query: a frustum (one plane may be crossed) and an overlap range, And and Or
    {
      const BoundingBox3D range{ { 30, 30, 30 }, { 70, 70, 70 } };
      std::vector<std::pair<Plane3D, bool>> fr;
      for (std::size_t i = 0; i < planes.size(); ++i)
        fr.emplace_back(planes[i], i == 0);
      const std::vector<OctreeBoxM::QueryCondition> conds = { OctreeBoxM::ByInFrustum(fr), OctreeBoxM::ByOverlaps(range) };
      struct
      {
        int32_t kind;
        uint32_t first, count, reserved;
        double tol;
      } oc[2] = { { OTG_COND_FRUSTUM, 0, uint32_t(planes.size()), 0, -1.0 }, { OTG_COND_RANGE_OVERLAP, 0, 1, 0, -1.0 } };
      const uint64_t off[2] = { 0, 2 };
      std::vector<unsigned char> cross(planes.size(), 0);
      cross[0] = 1;
      for (int orOp = 0; orOp < 2; ++orOp)
      {
        r = oro_query(ob, oc, off, 1, planes.data(), cross.data(), &range, orOp, -1.0);
        expect(orOp ? tb.Query<LogicalOperator::Or>(conds) : tb.Query<LogicalOperator::And>(conds), r, 0, orOp ? "Query<Or>" : "Query<And>");
        oro_res_free(r);
      }
    }
    // collisions: pairs flattened to ids
    auto flat = [](const std::vector<std::pair<EntityID, EntityID>>& p) {
      std::vector<uint32_t> v;
      for (auto [a, b] : p)
      {
        v.push_back(a);
        v.push_back(b);
      }
      return v;
    };
    r = oro_collide_self(ob, -1.0);
    expect(flat(tb.CollisionDetection()), r, 0, "CollisionDetection");
    oro_res_free(r);
    std::vector<BoundingBox3D> other(boxes.begin(), boxes.begin() + 5000);
    for (auto& b : other)
      for (int c = 0; c < 3; ++c)
      {
        b.Min[c] += 0.2;
        b.Max[c] += 0.2;
      }
    OctreeBoxM to(other, 6, std::nullopt, 12);
    void* oo = oro_create(0, 1, other.data(), other.size(), 6, nullptr, 12);
    r = oro_collide_pair(ob, oo, -1.0);
    expect(flat(OctreeBoxM::CollisionDetection(tb, to)), r, 0, "CollisionDetection(two trees)");
    oro_res_free(r);
    oro_destroy(oo);
  }
  oro_destroy(ob);
  // ---- regular (non-loose) boxes: OctreeBoxMs<false>
  {
    OctreeBoxMs<false> tr(boxes, 7, std::nullopt, 16);
    void* orr = oro_create(0, 2, boxes.data(), boxes.size(), 7, nullptr, 16);
    void* r = oro_range(orr, ranges.data(), nq, 1, -1.0);
    for (int q = 0; q < nq; ++q)
      expect(tr.RangeSearch(ranges[q], RangeSearchMode::Overlap), r, q, "RangeSearch (regular boxes)");
    oro_res_free(r);
    std::vector<uint32_t> flat;
    for (auto [a, b] : tr.CollisionDetection())
    {
      flat.push_back(a);
      flat.push_back(b);
    }
    r = oro_collide_self(orr, -1.0);
    expect(flat, r, 0, "CollisionDetection (regular boxes)");
    oro_res_free(r);
    oro_destroy(orr);
  }
  // ---- the Core form (non-owning): the entity span on Create and on every query
  {
    std::vector<Point3D> span1(pts.begin(), pts.begin() + 30000);
    OctreePoint tc(std::span<const Point3D>(span1), 8, std::nullopt, 20);
    // the span's tree, as the oracle builds it; kNN, range and pick of the Core type against it
    auto check_span = [&](std::span<const Point3D> span, const char* what) {
      void* oc = oro_create(0, 0, span.data(), span.size(), 8, nullptr, 20);
      void* r = oro_range(oc, ranges.data(), nq, 0, -1.0);
      for (int i = 0; i < nq; ++i)
        expect(tc.RangeSearch(ranges[i], span), r, i, what);
      oro_res_free(r);
      std::vector<uint32_t> k(nq, 7);
      r = oro_knn(oc, qp.data(), nq, k.data(), -1.0, -1.0);
      for (int i = 0; i < nq; ++i)
        expect(tc.GetNearestNeighbors(qp[i], 7, span), r, i, what);
      oro_res_free(r);
      r = oro_pick(oc, qp.data(), nq, -1.0);
      for (int i = 0; i < nq; ++i)
        expect(tc.PickSearch(qp[i], span), r, i, what);
      oro_res_free(r);
      oro_destroy(oc);
    };
    check_span(span1, "Core: the Create span");
    // another span (SpanChange::Rebuild, the default): the tree of that span
    std::vector<Point3D> span2(span1);
    for (std::size_t i = 0; i < span2.size(); i += 3)
      for (int c = 0; c < 3; ++c)
        span2[i][c] += 0.7 * N(rng);
    check_span(span2, "Core: another span");
    // the first span changed in place: uploaded again after NotifyEntitiesChanged
    for (std::size_t i = 1; i < span1.size(); i += 5)
      span1[i][0] += 1.3;
    tc.NotifyEntitiesChanged();
    check_span(span1, "Core: span changed in place");
    // SpanChange::KeepNodes: the nodes of the last Create stay and the new geometry is tested, as the
    // reference answers with a span other than its Create's (queries that test a fixed set of nodes)
    {
      OctreePoint tk(std::span<const Point3D>(span1), 8, std::nullopt, 20);
      tk.SetSpanChange(OctreePoint::SpanChange::KeepNodes);
      void* ok = oro_create(0, 0, span1.data(), span1.size(), 8, nullptr, 20);
      oro_set_entities(ok, span2.data(), span2.size());
      void* r = oro_range(ok, ranges.data(), nq, 0, -1.0);
      for (int i = 0; i < nq; ++i)
        expect(tk.RangeSearch(ranges[i], std::span<const Point3D>(span2)), r, i, "Core KeepNodes: RangeSearch");
      oro_res_free(r);
      r = oro_pick(ok, qp.data(), nq, -1.0);
      for (int i = 0; i < nq; ++i)
        expect(tk.PickSearch(qp[i], std::span<const Point3D>(span2)), r, i, "Core KeepNodes: PickSearch");
      oro_res_free(r);
      oro_destroy(ok);
      // a span of another size does not fit the nodes
      bool refused = false;
      try
      {
        tk.RangeSearch(ranges[0], std::span<const Point3D>(span1.data(), span1.size() - 1));
      }
      catch (const Error& e)
      {
        refused = e.status() == OTG_ERR_INVALID_ARGUMENT;
      }
      if (!refused)
      {
        std::printf("MISMATCH Core KeepNodes: a span of another size was not refused\n");
        ++g_fail;
      }
    }
    // bulk Insert: Managed Add and Core Insert of new points, against the oracle's Insert
    {
      std::vector<Point3D> base(pts.begin(), pts.begin() + 20000), add(pts.begin() + 20000, pts.begin() + 26000);
      for (std::size_t i = 0; i < add.size(); i += 2)
        add[i] = { 40.0 + 0.01 * N(rng), 60.0 + 0.01 * N(rng), 20.0 + 0.01 * N(rng) }; // a deep cluster
      // a given space, so that every new point lies inside it
      const BoundingBox3D space{ { 0.0, 0.0, 0.0 }, { 100.0, 100.0, 100.0 } };
      OctreePointM tm(base, 8, space, 20);
      OctreePoint ti(std::span<const Point3D>(base), 8, space, 20);
      void* oi = oro_create(0, 0, base.data(), base.size(), 8, &space, 20);
      const bool ok = oro_insert(oi, add.data(), add.size()) && tm.Add(std::span<const Point3D>(add)) &&
                      ti.Insert(std::span<const Point3D>(add), std::span<const Point3D>(base));
      if (!ok || tm.GetEntityCount() != base.size() + add.size() || tm.GetNodeCount() != ti.GetNodeCount())
      {
        std::printf("MISMATCH Insert: refused or counts differ\n");
        ++g_fail;
      }
      std::vector<Point3D> all(base);
      all.insert(all.end(), add.begin(), add.end());
      std::span<const Point3D> allSpan(all);
      void* r = oro_range(oi, ranges.data(), nq, 0, -1.0);
      for (int i = 0; i < nq; ++i)
      {
        expect(tm.RangeSearch(ranges[i]), r, i, "Managed Add: RangeSearch");
        expect(ti.RangeSearch(ranges[i], allSpan), r, i, "Core Insert: RangeSearch");
      }
      oro_res_free(r);
      std::vector<uint32_t> k(nq, 11);
      r = oro_knn(oi, qp.data(), nq, k.data(), -1.0, -1.0);
      for (int i = 0; i < nq; ++i)
      {
        expect(tm.GetNearestNeighbors(qp[i], 11), r, i, "Managed Add: GetNearestNeighbors");
        expect(ti.GetNearestNeighbors(qp[i], 11, allSpan), r, i, "Core Insert: GetNearestNeighbors");
      }
      oro_res_free(r);
      r = oro_pick(oi, add.data(), nq, -1.0);
      for (int i = 0; i < nq; ++i)
        expect(tm.PickSearch(add[i]), r, i, "Managed Add: PickSearch");
      oro_res_free(r);
      oro_destroy(oi);
      // a point outside the space: nothing inserted, its id in failedEntities
      const std::vector<Point3D> bad{ { 50.0, 50.0, 50.0 }, { 150.0, 50.0, 50.0 } };
      std::unordered_set<EntityID> failed;
      const std::size_t nodes = ti.GetNodeCount();
      if (tm.Add(std::span<const Point3D>(bad)) || ti.Insert(std::span<const Point3D>(bad), allSpan, nullptr, &failed) || failed.size() != 1 ||
          !failed.count(EntityID(all.size() + 1)) || ti.GetNodeCount() != nodes || tm.GetEntityCount() != all.size())
      {
        std::printf("MISMATCH Insert: a point outside the space was not refused\n");
        ++g_fail;
      }
    }
    // box trees: collisions with the span, and the two-tree form
    std::vector<BoundingBox3D> bspan(boxes.begin(), boxes.begin() + 8000);
    OctreeBox tbc(std::span<const BoundingBox3D>(bspan), 7, std::nullopt, 16);
    OctreeBox tbo;
    std::vector<BoundingBox3D> ospan(boxes.begin() + 8000, boxes.begin() + 12000);
    OctreeBox::Create(tbo, std::span<const BoundingBox3D>(ospan), 6, std::nullopt, 12);
    void* obo = oro_create(0, 1, ospan.data(), ospan.size(), 6, nullptr, 12);
    auto flat = [](const std::vector<std::pair<EntityID, EntityID>>& p) {
      std::vector<uint32_t> v;
      for (auto [a, b] : p)
      {
        v.push_back(a);
        v.push_back(b);
      }
      return v;
    };
    for (int round = 0; round < 2; ++round)
    {
      void* obc = oro_create(0, 1, bspan.data(), bspan.size(), 7, nullptr, 16);
      void* r = oro_collide_self(obc, -1.0);
      expect(flat(tbc.CollisionDetection(std::span<const BoundingBox3D>(bspan))), r, 0, "Core: CollisionDetection");
      oro_res_free(r);
      r = oro_collide_pair(obc, obo, -1.0);
      expect(flat(OctreeBox::CollisionDetection(tbc, std::span<const BoundingBox3D>(bspan), tbo, std::span<const BoundingBox3D>(ospan))), r, 0,
             "Core: CollisionDetection(two trees)");
      oro_res_free(r);
      oro_destroy(obc);
      // move some boxes of the first span in place: the next pass of the loop answers for the moved span
      for (std::size_t i = 0; i < bspan.size(); i += 4)
        for (int c = 0; c < 3; ++c)
        {
          bspan[i].Min[c] += 0.5;
          bspan[i].Max[c] += 0.5;
        }
      tbc.NotifyEntitiesChanged();
    }
    oro_destroy(obo);
  }
  if (g_fail)
    return 1;
  std::printf("OK\n");
  return 0;
}
