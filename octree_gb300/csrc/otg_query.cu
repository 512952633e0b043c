// otg_query.cu — data-parallel queries over a GPU tree.
//
// Plain kernels: one query per thread, FP64 (or the tree's scalar) arithmetic in the reference's
// operation order, explicit depth-first node stack. They prune with exactly the node tests of the
// reference (same node boxes, same predicates), so the id sets equal the reference's:
//   RangeSearch         core/ot_query.h:476-583
//   PickSearch          core/ot_query.h:425-466
//   FrustumCulling      core/ot_query.h:767-833
//   PlaneSearch         core/ot_query.h:612-636
//   PlanePositiveSegmentation core/ot_query.h:687-744
//   Query<And / Or>     core/ot_query.h:864-1026
//   GetNearestNeighbors core/ot_query.h:1208-1270
//   RayIntersectedAll   core/ot_query.h:1928-2022
//   RayIntersectedFirst core/ot_query.h:2035-2146
//   CollisionDetection  core/ot_query.h:1308-1497 (two trees), 1690-1914 (one tree)
//
// Results are appended as (query << 32 | id) items (plus a distance where the query has one),
// then ordered with stable radix sorts into CSR form: ids ascending per query, or by
// (distance, id) for kNN and rays, or (i, j) pairs ascending for collisions.
#include "otg_query.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

namespace otg
{

// ---------------------------------------------------------------- RangeSearch (plain)
template<typename T>
__global__ void __launch_bounds__(128) range_plain_kernel(TreeView<T> tv, const T* __restrict__ ranges, u32 nq, int mode, T tol, Appender out,
                                                          u32* err)
{
  using G = GeoD<T>;
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  T r[6];
  load_box(ranges + u64(q) * 6, r);
  // root shortcut (:488-511): the whole root box inside the range -> every entity id
  {
    T rb[6];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      rb[c] = tv.nodeBox[u64(root) * 6 + c];
      rb[3 + c] = tv.nodeBox[u64(root) * 6 + c] + tv.nodeBox[u64(root) * 6 + 3 + c];
    }
    if (G::range_contains_box(r, rb, tol))
    {
      const u32 nt = tv.qTree ? u32(tv.treeOff[root + 1] - tv.treeOff[root]) : tv.n;
      u64 pos = out.reserve(nt);
      for (u32 i = 0; i < nt; ++i)
        if (pos + i < out.capacity)
          out.items[pos + i] = (u64(q) << 32) | i;
      return;
    }
  }
  // zero-volume range -> empty (:514-519)
  T vol = T(1);
#pragma unroll
  for (int c = 0; c < 3; ++c)
    vol *= T(r[3 + c] - r[c]);
  if (vol <= T(0))
    return;
  T rmin[3], rsize[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
  {
    rmin[c] = r[c];
    rsize[c] = T(r[3 + c] - r[c]);
  }
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    T nmin[3], nsize[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      nmin[c] = nb[c];
      nsize[c] = nb[3 + c];
    }
    if (!G::overlap_by_min_point(rmin, rsize, nmin, nsize, tol))
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    if (G::range_contains_min_size(r, nmin, nsize, tol))
    {
      // whole subtree without entity tests (:549-567); the subtree is one run of sortedIds
      const u32 len = L.w - L.y;
      u64 pos = out.reserve(len);
      for (u32 i = 0; i < len; ++i)
        if (pos + i < out.capacity)
          out.items[pos + i] = (u64(q) << 32) | (tv.ids[L.y + i] - idBase);
      continue;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      bool ok;
      if (!tv.isBox)
        ok = G::box_contains_point(r, tv.geom + u64(e) * 3, tol);
      else
      {
        T b[6];
        load_box(tv.geom + u64(e) * 6, b);
        ok = (mode == OTG_RANGE_OVERLAP) ? (G::box_relation(r, b, tol) == -1) : G::contains_box_no_tol(r, b);
      }
      if (ok)
        out.put(q, (tv.ids[e] - idBase));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// ---------------------------------------------------------------- PickSearch (plain)
template<typename T>
__global__ void __launch_bounds__(128) pick_plain_kernel(TreeView<T> tv, const T* __restrict__ pts, u32 nq, T tol, Appender out, u32* err)
{
  using G = GeoD<T>;
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  T p[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    p[c] = pts[u64(q) * 3 + c];
  {
    T rb[6];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      rb[c] = tv.nodeBox[u64(root) * 6 + c];
      rb[3 + c] = tv.nodeBox[u64(root) * 6 + c] + tv.nodeBox[u64(root) * 6 + 3 + c];
    }
    if (!G::box_contains_point(rb, p, tol)) // :430-431 (DoesBoxContainPointAD box form)
      return;
  }
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    if (!G::node_contains_point(nb, nb + 3, p, tol))
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      bool ok = tv.isBox ? G::box_contains_point(tv.geom + u64(e) * 6, p, tol) : G::points_equal(tv.geom + u64(e) * 3, p, tol);
      if (ok)
        out.put(q, (tv.ids[e] - idBase));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// ---------------------------------------------------------------- FrustumCulling (plain)
template<typename T>
__global__ void __launch_bounds__(128) frustum_plain_kernel(TreeView<T> tv, const T* __restrict__ planes, u32 np, u32 nq, T tol, Appender out,
                                                            u32* err)
{
  using G = GeoD<T>;
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq || np == 0)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  const T* pl = planes + u64(q) * np * 4;
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    bool select = true;
    for (u32 i = 0; i < np; ++i) // :779-795 first Hit selects, first Negative prunes
    {
      int rel = G::box_plane(nb, nb + 3, pl[4 * i], pl + 4 * i + 1, tol);
      if (rel == 1)
        break;
      if (rel == 0)
      {
        select = false;
        break;
      }
    }
    if (!select)
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      bool neg = false;
      for (u32 i = 0; i < np && !neg; ++i)
      {
        int rel;
        if (tv.isBox)
        {
          const T* b = tv.geom + u64(e) * 6;
          T bsize[3] = { T(b[3] - b[0]), T(b[4] - b[1]), T(b[5] - b[2]) };
          rel = G::box_plane(b, bsize, pl[4 * i], pl + 4 * i + 1, tol);
        }
        else
          rel = G::point_plane(tv.geom + u64(e) * 3, pl[4 * i], pl + 4 * i + 1, tol);
        neg = rel == 0;
      }
      if (!neg)
        out.put(q, (tv.ids[e] - idBase));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// ---------------------------------------------------------------- PlaneSearch / PlanePositiveSegmentation (plain)
// One plane {origoDistance, nx, ny, nz} per query. PlaneSearch enters the nodes the plane hits and
// keeps the entities it hits; PlanePositiveSegmentation prunes negative nodes, takes a positive
// node's whole subtree untested and keeps the entities of hit nodes that are not negative.
template<typename T>
__global__ void __launch_bounds__(128) plane_plain_kernel(TreeView<T> tv, const T* __restrict__ planes, u32 nq, int positive, T tol, Appender out,
                                                          u32* err)
{
  using G = GeoD<T>;
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  const T* pl = planes + u64(q) * 4;
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    const int rel = G::box_plane(nb, nb + 3, pl[0], pl + 1, tol);
    if (positive ? rel == 0 : rel != 1)
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    if (positive && rel == 2)
    {
      // the whole subtree, untested (:711-726); a subtree is one run of sortedIds
      const u32 len = L.w - L.y;
      u64 pos = out.reserve(len);
      for (u32 i = 0; i < len; ++i)
        if (pos + i < out.capacity)
          out.items[pos + i] = (u64(q) << 32) | (tv.ids[L.y + i] - idBase);
      continue;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      int er; // :586-602 GetEntityPlaneRelation
      if (tv.isBox)
      {
        const T* b = tv.geom + u64(e) * 6;
        T bsize[3] = { T(b[3] - b[0]), T(b[4] - b[1]), T(b[5] - b[2]) };
        er = G::box_plane(b, bsize, pl[0], pl + 1, tol);
      }
      else
        er = G::point_plane(tv.geom + u64(e) * 3, pl[0], pl + 1, tol);
      if (positive ? er != 0 : er == 1)
        out.put(q, (tv.ids[e] - idBase));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// ---------------------------------------------------------------- Query<And / Or> (plain)
// A node is entered when its conditions pass (all under And, any under Or), and its own entities are
// kept when theirs pass; there is no whole-subtree shortcut, as in the reference.
template<typename T>
__global__ void __launch_bounds__(128) query_plain_kernel(TreeView<T> tv, QueryProgram<T> qp, u32 nq, T tol, Appender out, u32* err)
{
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  const u32 W = tv.isBox ? 6 : 3;
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    if (!cond_combine(qp, q, err, [&](const QueryCond& c) { return cond_node(qp, c, nb, tol); }))
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      const T* g = tv.geom + u64(e) * W;
      if (cond_combine(qp, q, err, [&](const QueryCond& c) { return cond_entity(qp, c, g, tv.isBox != 0, tol); }))
        out.put(q, (tv.ids[e] - idBase));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// ---------------------------------------------------------------- kNN (plain)

// Pass 1: the k-th smallest distance d_k (points) -> F = U(d_k), the reference's final
// farthestEntityDistance. Box trees keep the reference's optimistic/pessimistic pair:
// the pessimistic (minMax) k-th distance sets F, entities qualify by their min distance.
// KMAX: the heap's capacity, a bucket at or above every k of the launch (8, 16, ..., 256), so a
// query with small k keeps a small heap.
template<typename T, int KMAX>
__global__ void __launch_bounds__(128) knn_threshold_kernel(TreeView<T> tv, const T* __restrict__ pts, u32 nq, const u32* __restrict__ kArr, u32 kAll,
                                                            T F0, T tol, T* __restrict__ Fout, u32* err)
{
  using G = GeoD<T>;
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  u32 k = kArr ? kArr[q] : kAll;
  if (k == 0) // ot_query.h:1217-1219: no neighbour requested -> empty result (no distance is below 0)
  {
    Fout[q] = T(0);
    return;
  }
  if (k > u32(KMAX))
  {
    atomicOr(err, kErrCapacity);
    k = KMAX;
  }
  T p[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    p[c] = pts[u64(q) * 3 + c];
  T heap[KMAX]; // max-heap of the k smallest (pessimistic) distances
  u32 hs = 0;
  T F = F0;
  u32 stack[kStack];
  T sdist[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp] = root;
  sdist[sp++] = G::wall_distance(p, tv.nodeBox + u64(root) * 6, tv.nodeBox + u64(root) * 6 + 3);
  while (sp > 0 && k > 0)
  {
    --sp;
    const u32 node = stack[sp];
    if (sdist[sp] >= F)
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      // a broken node record: the call fails; the threshold is still written (0: no entity
      // qualifies), so the collect pass never reads an unwritten value
      atomicOr(err, kErrStack);
      F = T(0);
      break;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      T dmin, dmm;
      if (tv.isBox)
        G::min_max_distance(p, tv.geom + u64(e) * 6, tol, dmin, dmm);
      else
        dmin = dmm = G::distance(p, tv.geom + u64(e) * 3);
      if (dmin >= F)
        continue;
      if (hs < k)
      {
        // sift up
        u32 i = hs++;
        while (i > 0)
        {
          u32 par = (i - 1) >> 1;
          if (!(heap[par] < dmm))
            break;
          heap[i] = heap[par];
          i = par;
        }
        heap[i] = dmm;
        if (hs == k)
          F = upper_tol(heap[0], tol); // :1123-1128 (heapify sets F unconditionally)
      }
      else if (dmm < heap[0])
      {
        // replace the max, sift down
        u32 i = 0;
        for (;;)
        {
          u32 l = 2 * i + 1, r = l + 1, m = i;
          T vm = dmm;
          if (l < hs && vm < heap[l])
          {
            m = l;
            vm = heap[l];
          }
          if (r < hs && vm < heap[r])
          {
            m = r;
            vm = heap[r];
          }
          if (m == i)
            break;
          heap[i] = heap[m];
          i = m;
        }
        heap[i] = dmm;
        T lim = upper_tol(heap[0], tol);
        if (lim < F)
          F = lim;
      }
    }
    // children, nearest popped first
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      break;
    }
    const int base = sp;
    for (u32 c = 0; c < cc; ++c)
    {
      const T* nb = tv.nodeBox + u64(fc + c) * 6;
      T w = G::wall_distance(p, nb, nb + 3);
      if (w >= F)
        continue;
      // insertion keeping [base, sp) sorted by descending distance
      int j = sp++;
      while (j > base && sdist[j - 1] < w)
      {
        sdist[j] = sdist[j - 1];
        stack[j] = stack[j - 1];
        --j;
      }
      sdist[j] = w;
      stack[j] = fc + c;
    }
  }
  Fout[q] = F;
}

// Pass 2: every entity with (min) distance < F, appended with its distance.
template<typename T>
__global__ void __launch_bounds__(128) knn_collect_kernel(TreeView<T> tv, const T* __restrict__ pts, u32 nq, const T* __restrict__ Fin, T tol, Appender out,
                                                          u32* err)
{
  using G = GeoD<T>;
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  const T F = Fin[q];
  T p[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    p[c] = pts[u64(q) * 3 + c];
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    if (G::wall_distance(p, nb, nb + 3) >= F)
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      T d = entity_distance(tv, e, p, tol);
      if (d < F)
        out.put(q, (tv.ids[e] - idBase), double(d));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// The heap bucket of the plain kNN threshold pass for a largest k of kMax.
static int knn_heap_bucket(u32 kMax)
{
  int b = 8;
  while (b < kKnnMaxK && u32(b) < kMax)
    b *= 2;
  return b;
}

template<typename T>
static void launch_knn_threshold(int bucket, u32 blocks, cudaStream_t st, TreeView<T> tv, const T* pts, u32 nq, const u32* kArr, u32 kAll, T F0,
                                 T tol, T* Fout, u32* err)
{
  switch (bucket)
  {
  case 8: knn_threshold_kernel<T, 8><<<blocks, 128, 0, st>>>(tv, pts, nq, kArr, kAll, F0, tol, Fout, err); break;
  case 16: knn_threshold_kernel<T, 16><<<blocks, 128, 0, st>>>(tv, pts, nq, kArr, kAll, F0, tol, Fout, err); break;
  case 32: knn_threshold_kernel<T, 32><<<blocks, 128, 0, st>>>(tv, pts, nq, kArr, kAll, F0, tol, Fout, err); break;
  case 64: knn_threshold_kernel<T, 64><<<blocks, 128, 0, st>>>(tv, pts, nq, kArr, kAll, F0, tol, Fout, err); break;
  case 128: knn_threshold_kernel<T, 128><<<blocks, 128, 0, st>>>(tv, pts, nq, kArr, kAll, F0, tol, Fout, err); break;
  default: knn_threshold_kernel<T, kKnnMaxK><<<blocks, 128, 0, st>>>(tv, pts, nq, kArr, kAll, F0, tol, Fout, err); break;
  }
}

// largest value of a device array (0 for n = 0) into *out, which the caller zeroed
__global__ void max_u32_kernel(const u32* __restrict__ a, u64 n, u32* __restrict__ out)
{
  u32 m = 0;
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
    m = max(m, a[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m)
    atomicMax(out, m);
}

// ---------------------------------------------------------------- rays (plain)
template<typename T>
__device__ __forceinline__ bool entity_hit(const TreeView<T>& tv, const RayD<T>& ray, u32 e, T& en, T& ex)
{
  return tv.isBox ? ray.hit_box(tv.geom + u64(e) * 6, en, ex) : ray.hit_point(tv.geom + u64(e) * 3, en, ex);
}

// RayIntersectedAll: DFS over nodes hit by the ray; entities hit with enter <= maxDist (or maxDist == 0)
template<typename T>
__global__ void __launch_bounds__(128) ray_all_plain_kernel(TreeView<T> tv, const T* __restrict__ rays, u32 nq, T tol, T tolInc, T maxDist, Appender out,
                                                            u32* err)
{
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  RayD<T> ray;
  ray.make(rays + u64(q) * 6, rays + u64(q) * 6 + 3, tol, tolInc);
  if (!ray.valid)
    return;
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    T en, ex;
    if (!ray.hit_node(nb, nb + 3, en, ex))
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      if (!entity_hit(tv, ray, e, en, ex))
        continue;
      if (!(maxDist == T(0) || en <= maxDist))
        continue;
      out.put(q, (tv.ids[e] - idBase), double(en));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// RayIntersectedFirst, pass 1: M = (1 + tolInc) * (smallest exit among hits with enter <= maxDist) + tol'
// (ot_query.h:2093-2103), never above maxDist; pass 2 collects every hit with enter <= M.
template<typename T>
__global__ void __launch_bounds__(128) ray_first_threshold_kernel(TreeView<T> tv, const T* __restrict__ rays, u32 nq, T tol, T tolInc, T maxDist,
                                                                  T* __restrict__ Mout, u32* err)
{
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  RayD<T> ray;
  ray.make(rays + u64(q) * 6, rays + u64(q) * 6 + 3, tol, tolInc);
  T M = maxDist;
  if (!ray.valid)
  {
    Mout[q] = -Lim<T>::max();
    return;
  }
  const T applied = tol == T(0) ? Lim<T>::eps() : tol;
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    T en, ex;
    if (!ray.hit_node(nb, nb + 3, en, ex) || en > M)
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      if (!entity_hit(tv, ray, e, en, ex))
        continue;
      if (en > M || ex >= M)
        continue;
      M = (T(1) + tolInc) * ex + applied;
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      break;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
  Mout[q] = M;
}

template<typename T>
__global__ void __launch_bounds__(128) ray_first_collect_kernel(TreeView<T> tv, const T* __restrict__ rays, u32 nq, T tol, T tolInc, const T* __restrict__ Min,
                                                                Appender out, u32* err)
{
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const u32 root = query_root(tv, q);
  const u32 idBase = id_base(tv, root);
  RayD<T> ray;
  ray.make(rays + u64(q) * 6, rays + u64(q) * 6 + 3, tol, tolInc);
  if (!ray.valid)
    return;
  const T M = Min[q];
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = root;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    T en, ex;
    if (!ray.hit_node(nb, nb + 3, en, ex) || en > M)
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      if (!entity_hit(tv, ray, e, en, ex))
        continue;
      if (en > M)
        continue;
      out.put(q, (tv.ids[e] - idBase), double(en));
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// ---------------------------------------------------------------- collision (plain)
// One thread per query box; tree B's node MBRs (exact min / max corners) prune conservatively
// and every candidate pair is decided by GetBoxRelation == Overlapped (general.h:262-294), the
// predicate of both reference paths. selfMode: only pairs with idB > idA are reported.
template<typename T>
__global__ void __launch_bounds__(128) collide_plain_kernel(TreeView<T> ta, TreeView<T> tb, T tol, int selfMode, Appender out, u32* err)
{
  using G = GeoD<T>;
  const u32 i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ta.n)
    return;
  T a[6];
  load_box(ta.geom + u64(i) * 6, a);
  const u32 idA = ta.ids[i];
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = 0;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nmin = tb.nodeBox + u64(node) * 6;
    const T* nmax = tb.nodeMax + u64(node) * 3;
    // GetBoxRelation can only answer "overlapped" when neither max + tol < other min (in the
    // scalar's arithmetic); every box of the node lies inside its exact MBR, so this prune never
    // drops a pair the predicate accepts
    bool disjoint = false;
#pragma unroll
    for (int c = 0; c < 3; ++c)
      disjoint |= (T(a[3 + c] + tol) < nmin[c]) || (T(nmax[c] + tol) < a[c]);
    if (disjoint)
      continue;
    const uint4 L = tb.link[node];
    if (L.z > tb.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      const u32 idB = tb.ids[e];
      if (selfMode && idB <= idA)
        continue;
      T b[6];
      load_box(tb.geom + u64(e) * 6, b);
      if (G::box_relation(a, b, tol) == -1)
        out.put(i, e); // sorted positions; collide_filter_kernel maps them to ids
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tb.nNodes) || ++visits > tb.nNodes)
    {
      atomicOr(err, kErrStack);
      return;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
}

// ---------------------------------------------------------------- collision structure filter
// The reference compares an overlapping pair only if its tree walk reaches the pair's two nodes,
// and that walk prunes with AreBoxesOverlappingByMinPoint on node boxes (min, min + size) with the
// tolerance. For strictly overlapping boxes those tests pass except at rounding level, which in
// float trees with coordinates far above the tolerance does happen. This filter applies the walk's
// conditions to every candidate pair exactly:
//   same node          InsertCollidedEntitiesInsideNode: always compared (ot_query.h:1518-1561)
//   ancestor entity p   InsertCollidedEntitiesWithParents: p.minX <= node.Box.Max[0] and
//                       AreBoxesOverlappingByMinPoint(node, p) (ot_query.h:1563-1653)
//   sibling subtrees    two-tree walk from the sibling pair (first pair untested), then every
//                       descent pair tested (ot_query.h:1308-1458, called at :1672-1684)
//   two trees           the same walk from the two roots (ot_query.h:1462-1485)
template<typename T>
struct StructTree
{
  const T* nodeBox;
  const u32* owner;
  const u32* parent;
  const unsigned char* depth;
  const T* geom;
  const u32* ids;
  const uint4* link;
};

template<typename T>
__device__ __forceinline__ int ancestors(const StructTree<T>& t, u32 x, u32* anc)
{
  int d = t.depth[x];
  if (d > 20)
    d = 20;
  anc[d] = x;
  for (int k = d; k > 0; --k)
    anc[k - 1] = t.parent[anc[k]];
  return d;
}

template<typename T>
__device__ __forceinline__ bool node_overlap(const StructTree<T>& ta, u32 a, const StructTree<T>& tb, u32 b, T tol)
{
  const T* na = ta.nodeBox + u64(a) * 6;
  const T* nb = tb.nodeBox + u64(b) * 6;
  return GeoD<T>::overlap_by_min_point(na, na + 3, nb, nb + 3, tol);
}

template<typename T>
__device__ __forceinline__ bool with_parent_condition(const StructTree<T>& t, u32 node, const T* p, T tol)
{
  const T* nb = t.nodeBox + u64(node) * 6;
  const T boxMax0 = nb[0] + nb[3];
  if (p[0] > boxMax0)
    return false;
  T psize[3] = { T(p[3] - p[0]), T(p[4] - p[1]), T(p[5] - p[2]) };
  return GeoD<T>::overlap_by_min_point(nb, nb + 3, p, psize, tol);
}

// The sweep-and-prune loops (ot_query.h:1367-1418, 1581-1650) visit, for an outer entity o, the
// inner entities of a node sorted by min-x starting at the first one whose max-x >= o.minX. An
// inner entity whose box ends before o starts is therefore tested only when an inner entity
// sorted before it (min-x, then id) reaches o.minX. GetBoxRelation can call such a pair
// overlapping when the gap is under one ulp but above the tolerance (the tolerance addition
// rounds up to the other coordinate).
template<typename T>
__device__ __forceinline__ bool sweep_reaches(const StructTree<T>& t, u32 innerNode, u32 innerPos, T outerMinX)
{
  const uint4 L = t.link[innerNode];
  const T* g = t.geom + u64(innerPos) * 6;
  const T mx = g[0];
  const u32 id = t.ids[innerPos];
  for (u32 q = L.y; q < L.z; ++q)
  {
    const T* h = t.geom + u64(q) * 6;
    const bool before = h[0] < mx || (h[0] == mx && t.ids[q] < id);
    if (before && h[3] >= outerMinX)
      return true;
  }
  return false;
}

// two-tree rules for outer (left) entity o and inner (right) entity at position ip in tree ti
template<typename T>
__device__ __forceinline__ bool sweep_pair(const T* o, const StructTree<T>& ti, u32 ip)
{
  const T* r = ti.geom + u64(ip) * 6;
  if (o[3] < r[0]) // the inner loop breaks at the first inner min-x above o.maxX
    return false;
  if (r[3] < o[0])
    return ti.owner[ip] != kNoOwner && sweep_reaches(ti, ti.owner[ip], ip, o[0]);
  return true;
}

template<typename T>
__global__ void __launch_bounds__(128) collide_filter_kernel(StructTree<T> A, StructTree<T> B, int selfMode, const u64* __restrict__ pairs, u64 m, T tol,
                                                             u64* __restrict__ keys, unsigned long long* rejected)
{
  for (u64 idx = blockIdx.x * u64(blockDim.x) + threadIdx.x; idx < m; idx += u64(gridDim.x) * blockDim.x)
  {
    const u64 it = pairs[idx];
    const u32 i = u32(it >> 32), j = u32(it);
    const u32 xa = A.owner[i], xb = B.owner[j];
    const T* ga = A.geom + u64(i) * 6;
    const T* gb = B.geom + u64(j) * 6;
    u32 ancA[21], ancB[21];
    bool keep = true;
    if (xa == kNoOwner || xb == kNoOwner)
      keep = false; // an entity in no node reachable from the root is in no pair of the reference's walk
    else if (!selfMode)
    {
      // CollisionDetection(left = A, right = B): node-pair walk from the roots, then the sweep
      keep = sweep_pair(ga, B, j);
      const int da = ancestors(A, xa, ancA);
      const int db = ancestors(B, xb, ancB);
      for (int k = 1; k <= max(da, db) && keep; ++k)
        keep = node_overlap(A, ancA[min(k, da)], B, ancB[min(k, db)], tol);
    }
    else if (xa == xb)
    {
      // InsertCollidedEntitiesInsideNode: ordered by (min-x, id), the later one must start
      // before the earlier one ends
      const bool aFirst = ga[0] < gb[0] || (ga[0] == gb[0] && A.ids[i] < A.ids[j]);
      keep = aFirst ? !(ga[3] < gb[0]) : !(gb[3] < ga[0]);
    }
    else
    {
      const int da = ancestors(A, xa, ancA);
      const int db = ancestors(A, xb, ancB);
      int dn = 0;
      while (dn + 1 <= min(da, db) && ancA[dn + 1] == ancB[dn + 1])
        ++dn;
      if (dn == da || dn == db)
      {
        // InsertCollidedEntitiesWithParents: node entity e (deeper node x) against ancestor entity p
        const bool aDeeper = dn == db ? true : false;
        const u32 x = aDeeper ? xa : xb;
        const u32 ep = aDeeper ? i : j;
        const T* e = aDeeper ? ga : gb;
        const T* p = aDeeper ? gb : ga;
        keep = with_parent_condition(A, x, p, tol);
        if (keep && p[3] < e[0])
          keep = false;
        if (keep && e[3] < p[0])
          keep = sweep_reaches(A, x, ep, p[0]);
      }
      else
      {
        // sibling sub-trees (ot_query.h:1672-1684): two-tree walk from (c1, c2), the earlier
        // child being the left tree; the first pair is not tested
        const bool aLeft = ancA[dn + 1] < ancB[dn + 1];
        keep = aLeft ? sweep_pair(ga, A, j) : sweep_pair(gb, A, i);
        for (int k = dn + 2; k <= max(da, db) && keep; ++k)
          keep = node_overlap(A, ancA[min(k, da)], A, ancB[min(k, db)], tol);
      }
    }
    u32 idA = A.ids[i], idB = B.ids[j];
    if (selfMode && idA > idB)
    {
      u32 t = idA;
      idA = idB;
      idB = t;
    }
    keys[idx] = keep ? ((u64(idA) << 32) | idB) : ~0ull;
    if (!keep)
      atomicAdd(rejected, 1ull);
  }
}

// ---------------------------------------------------------------- result finishing
// items (query << idBits | id) into query and id arrays
__global__ void split_items_kernel(const u64* __restrict__ items, const u32* __restrict__ perm, u64 m, u32* __restrict__ qOut, u32* __restrict__ idOut,
                                   u32 idBits = 32)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
  {
    u64 it = items[perm ? perm[i] : i];
    if (qOut)
      qOut[i] = u32(it >> idBits);
    idOut[i] = u32(it & ((u64(1) << idBits) - 1));
  }
}
// items (query << 32 | id) repacked as (query << idBits | id), so that their sort takes only the
// bits that queries and ids use
__global__ void pack_items_kernel(u64* __restrict__ items, u64 m, u32 idBits)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
  {
    const u64 it = items[i];
    items[i] = ((it >> 32) << idBits) | (it & 0xffffffffull);
  }
}
__global__ void gather_u64_kernel(const u64* __restrict__ src, const u32* __restrict__ perm, u64 m, u64* __restrict__ dst)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
    dst[i] = src[perm[i]];
}
__global__ void gather_dist_bits_kernel(const double* __restrict__ d, const u32* __restrict__ perm, u64 m, u64* __restrict__ dst)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
    dst[i] = u64(__double_as_longlong(d[perm[i]])); // distances are >= 0: bit order == value order
}
__global__ void gather_qid_kernel(const u64* __restrict__ items, const u32* __restrict__ perm, u64 m, u32* __restrict__ dst)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
    dst[i] = u32(items[perm[i]] >> 32);
}
__global__ void gather_final_kernel(const u64* __restrict__ items, const double* __restrict__ d, const u32* __restrict__ perm, u64 m,
                                    u32* __restrict__ idOut, double* __restrict__ dOut)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
  {
    u32 p = perm[i];
    idOut[i] = u32(items[p]);
    if (dOut)
      dOut[i] = d[p];
  }
}
// offsets[q] = first position whose query id >= q, from sorted query ids
__global__ void offsets_kernel(const u32* __restrict__ qid, u64 m, u64 nq, u64* __restrict__ offsets)
{
  for (u64 q = blockIdx.x * u64(blockDim.x) + threadIdx.x; q <= nq; q += u64(gridDim.x) * blockDim.x)
  {
    u64 lo = 0, hi = m;
    while (lo < hi)
    {
      u64 mid = (lo + hi) >> 1;
      if (u64(qid[mid]) < q)
        lo = mid + 1;
      else
        hi = mid;
    }
    offsets[q] = lo;
  }
}
__global__ void iota_kernel(u32* v, u64 m)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
    v[i] = u32(i);
}
__global__ void item_ids_kernel(const u64* __restrict__ items, u64 m, u32* __restrict__ dst)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
    dst[i] = u32(items[i]);
}

struct Collected
{
  // count: four words read back together: the item count, the filter's tests, the undecided tests,
  // and the error bits (the low half of the fourth)
  TmpBuf items, dist, count;
  u64 m = 0;
  u64 tests = 0, rechecks = 0;
  u32* errp() const { return reinterpret_cast<u32*>(count.as<unsigned long long>() + 3); }
};

static int status_of(u32 h)
{
  if (h & kErrStack)
  {
    set_error("traversal stack bound exceeded");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (h & kErrTimeout)
  {
    set_error("a bounded device wait ran out");
    return OTG_ERR_TIMEOUT;
  }
  if (h & kErrCapacity)
  {
    set_error("k above the supported maximum of 256");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (h & kErrArgument)
  {
    set_error("a query condition names a plane or box outside the given arrays, or an unknown kind");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  return OTG_OK;
}

// Runs launch(appender) until the append buffer was large enough; items end in c.items.
template<typename F>
static int collect(Collected& c, bool withDist, u64 guess, F&& launch, cudaStream_t st)
{
  cudaError_t e;
  if ((e = c.count.ensure(sizeof(unsigned long long) * 4, st)))
    return cuda_status(e, "allocating counters");
  u64 cap = std::max<u64>(guess, 1024);
  for (int attempt = 0; attempt < 3; ++attempt)
  {
    if ((e = c.items.ensure(sizeof(u64) * cap, st)) || (withDist && (e = c.dist.ensure(sizeof(double) * cap, st))))
      return cuda_status(e, "allocating result buffer");
    cudaMemsetAsync(c.count.p, 0, sizeof(unsigned long long) * 4, st);
    Appender a{ c.items.as<u64>(), withDist ? c.dist.as<double>() : nullptr, c.count.as<unsigned long long>(), cap };
    launch(a, c.errp());
    if ((e = cudaGetLastError()))
      return cuda_status(e, "launching query");
    unsigned long long h[4] = { 0, 0, 0, 0 };
    e = cudaMemcpyAsync(h, c.count.p, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (!e)
      e = cudaStreamSynchronize(st);
    if (e)
      return cuda_status(e, "running query");
    const unsigned long long m = h[0];
    c.tests = h[1];
    c.rechecks = h[2];
    if (int rc = status_of(u32(h[3])))
      return rc;
    if (m <= cap)
    {
      c.m = m;
      return OTG_OK;
    }
    cap = m + m / 8 + 1024;
  }
  set_error("result buffer sizing did not converge");
  return OTG_ERR_OUT_OF_MEMORY;
}

// ---- canonical order of (query, id) results by counting: each query's run, sorted by one warp
// items (query << 32 | id): the count of every query and each item's slot in its query's run
// (the lanes of a warp that hold the same query take their slots with one atomic)
__global__ void query_slots_kernel(const u64* __restrict__ items, u64 m, u32* __restrict__ cnt, u32* __restrict__ slot)
{
  const u32 lane = threadIdx.x & 31;
  const u64 stride = u64(gridDim.x) * blockDim.x;
  for (u64 base = blockIdx.x * u64(blockDim.x) + (threadIdx.x & ~31u); base < m; base += stride)
  {
    const u64 i = base + lane;
    const bool v = i < m;
    const u32 q = v ? u32(items[i] >> 32) : 0xffffffffu;
    const u32 peers = __match_any_sync(~0u, q);
    const int leader = __ffs(int(peers)) - 1;
    u32 b = 0;
    if (v && int(lane) == leader)
      b = atomicAdd(&cnt[q], u32(__popc(peers)));
    b = __shfl_sync(~0u, b, leader);
    if (v)
      slot[i] = b + __popc(peers & ((1u << lane) - 1u));
  }
}
__global__ void query_scatter_kernel(const u64* __restrict__ items, const u32* __restrict__ slot, u64 m, const u64* __restrict__ off, u32* __restrict__ ids)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
  {
    const u64 it = items[i];
    ids[off[u32(it >> 32)] + slot[i]] = u32(it);
  }
}
// One warp per query sorts its run of ids ascending: up to 32 in registers, up to kRunSortMax in
// shared memory (bitonic networks, padded with ~0); longer runs are only counted in *longRuns (the
// caller then orders the whole result another way).
constexpr u32 kRunSortMax = 1024;
constexpr int kRunSortWarps = 8;
__global__ void __launch_bounds__(kRunSortWarps * 32) run_sort_kernel(const u64* __restrict__ off, u64 nq, u32* __restrict__ ids, u32* __restrict__ longRuns)
{
  __shared__ u32 buf[kRunSortWarps][kRunSortMax];
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const u64 warps = u64(gridDim.x) * kRunSortWarps;
  for (u64 q = u64(blockIdx.x) * kRunSortWarps + w; q < nq; q += warps)
  {
    const u64 b = off[q];
    const u32 len = u32(off[q + 1] - b);
    if (len <= 1)
      continue;
    if (len > kRunSortMax)
    {
      if (lane == 0)
        atomicAdd(longRuns, 1u);
      continue;
    }
    if (len <= 32)
    {
      u32 v = lane < len ? ids[b + lane] : ~0u;
#pragma unroll
      for (u32 k = 2; k <= 32; k <<= 1)
#pragma unroll
        for (u32 j = k >> 1; j > 0; j >>= 1)
        {
          const u32 o = __shfl_xor_sync(~0u, v, j);
          const bool up = (lane & k) == 0, lower = (lane & j) == 0;
          v = (lower == up) ? min(v, o) : max(v, o);
        }
      if (lane < len)
        ids[b + lane] = v;
      continue;
    }
    u32 P = 64;
    while (P < len)
      P <<= 1;
    u32* s = buf[w];
    for (u32 i = lane; i < P; i += 32)
      s[i] = i < len ? ids[b + i] : ~0u;
    __syncwarp();
    for (u32 k = 2; k <= P; k <<= 1)
      for (u32 j = k >> 1; j > 0; j >>= 1)
      {
        for (u32 i = lane; i < P; i += 32)
        {
          const u32 x = i ^ j;
          if (x > i)
          {
            const u32 a = s[i], c = s[x];
            if ((a > c) == ((i & k) == 0))
            {
              s[i] = c;
              s[x] = a;
            }
          }
        }
        __syncwarp();
      }
    for (u32 i = lane; i < len; i += 32)
      ids[b + i] = s[i];
    __syncwarp();
  }
}

// CSR result with ids ascending per query; ids are below idLimit
static int finish_sorted_ids(Collected& c, u64 nq, ResultState& r, cudaStream_t st, u64 idLimit = u64(1) << 32)
{
  const u64 m = c.m;
  r.nq = nq;
  r.nids = m;
  r.hasDist = false;
  cudaError_t e;
  if ((e = result_alloc(r, sizeof(u64) * (nq + 1), sizeof(u32) * std::max<u64>(m, 1), 0, st)))
    return cuda_status(e, "allocating result");
  if (m == 0)
    return cuda_status(cudaMemsetAsync(r.offsets.p, 0, sizeof(u64) * (nq + 1), st), "result offsets");
  // runs longer than kRunSortMax on average certainly include long ones: straight to the radix sort
  // (counting them would also put every item's atomic on a few counters)
  if (m < (u64(1) << 32) && nq < (u64(1) << 31) && m <= u64(kRunSortMax) * nq)
  {
    // counting order: counts and slots, offsets, ids into their runs, each run sorted by a warp
    TmpBuf cnt, slot, tileSums, longRuns;
    const u64 tiles = (nq + kScanTile - 1) / kScanTile;
    if ((e = cnt.ensure(sizeof(u32) * nq, st)) || (e = slot.ensure(sizeof(u32) * m, st)) || (e = tileSums.ensure(sizeof(u64) * (tiles + 1), st)) ||
        (e = longRuns.ensure(sizeof(u32), st)))
      return cuda_status(e, "allocating the result order");
    cudaMemsetAsync(cnt.p, 0, sizeof(u32) * nq, st);
    cudaMemsetAsync(longRuns.p, 0, sizeof(u32), st);
    query_slots_kernel<<<blocks_for(m), 256, 0, st>>>(c.items.as<u64>(), m, cnt.as<u32>(), slot.as<u32>());
    scan_reduce_kernel<<<u32(tiles), kScanThreads, 0, st>>>(cnt.as<u32>(), nq, tileSums.as<u64>());
    scan_tiles_kernel<<<1, kScanThreads, 0, st>>>(tileSums.as<u64>(), tiles);
    scan_apply_kernel<<<u32(tiles), kScanThreads, 0, st>>>(cnt.as<u32>(), nq, tileSums.as<u64>(), r.offsets.as<u64>());
    query_scatter_kernel<<<blocks_for(m), 256, 0, st>>>(c.items.as<u64>(), slot.as<u32>(), m, r.offsets.as<u64>(), r.ids.as<u32>());
    run_sort_kernel<<<u32(std::min<u64>((nq + kRunSortWarps - 1) / kRunSortWarps, 152 * 8)), kRunSortWarps * 32, 0, st>>>(r.offsets.as<u64>(), nq,
                                                                                                                          r.ids.as<u32>(), longRuns.as<u32>());
    u32 hl = 0;
    if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(&hl, longRuns.p, sizeof(u32), cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
      return cuda_status(e, "finishing result");
    if (hl == 0)
      return OTG_OK;
    // some query holds more than kRunSortMax ids: the whole result by radix sort instead (the items
    // are unchanged)
  }
  TmpBuf vals, qid;
  if ((e = vals.ensure(sizeof(u32) * m, st)) || (e = qid.ensure(sizeof(u32) * m, st)))
    return cuda_status(e, "allocating sort values");
  const u32 idBits = std::min<u32>(32, std::max<u32>(1, bit_count(std::max<u64>(idLimit, 1) - 1)));
  if (idBits < 32)
    pack_items_kernel<<<blocks_for(m), 256, 0, st>>>(c.items.as<u64>(), m, idBits);
  if (int rc = sort_pairs_u64(c.items.as<u64>(), vals.as<u32>(), m, idBits + bit_count(nq), st, c.errp()))
    return rc;
  split_items_kernel<<<blocks_for(m), 256, 0, st>>>(c.items.as<u64>(), nullptr, m, qid.as<u32>(), r.ids.as<u32>(), idBits);
  offsets_kernel<<<blocks_for(nq + 1), 256, 0, st>>>(qid.as<u32>(), m, nq, r.offsets.as<u64>());
  e = cudaStreamSynchronize(st);
  return cuda_status(e ? e : cudaGetLastError(), "finishing result");
}

// CSR result ordered by (query, distance, id): three stable radix sorts (id, distance, query)
static int finish_by_distance(Collected& c, u64 nq, u64 nEntities, ResultState& r, cudaStream_t st)
{
  const u64 m = c.m;
  r.nq = nq;
  r.nids = m;
  r.hasDist = true;
  cudaError_t e;
  if ((e = result_alloc(r, sizeof(u64) * (nq + 1), sizeof(u32) * std::max<u64>(m, 1), sizeof(double) * std::max<u64>(m, 1), st)))
    return cuda_status(e, "allocating result");
  if (m == 0)
    return cuda_status(cudaMemsetAsync(r.offsets.p, 0, sizeof(u64) * (nq + 1), st), "result offsets");
  TmpBuf perm, k32, k64;
  if ((e = perm.ensure(sizeof(u32) * m, st)) || (e = k32.ensure(sizeof(u32) * m, st)) || (e = k64.ensure(sizeof(u64) * m, st)))
    return cuda_status(e, "allocating sort buffers");
  u32* err = c.errp();
  iota_kernel<<<blocks_for(m), 256, 0, st>>>(perm.as<u32>(), m);
  item_ids_kernel<<<blocks_for(m), 256, 0, st>>>(c.items.as<u64>(), m, k32.as<u32>());
  if (int rc = sort_pairs_u32(k32.as<u32>(), perm.as<u32>(), m, bit_count(nEntities), st, err))
    return rc;
  gather_dist_bits_kernel<<<blocks_for(m), 256, 0, st>>>(c.dist.as<double>(), perm.as<u32>(), m, k64.as<u64>());
  if (int rc = sort_pairs_u64(k64.as<u64>(), perm.as<u32>(), m, 64, st, err))
    return rc;
  gather_qid_kernel<<<blocks_for(m), 256, 0, st>>>(c.items.as<u64>(), perm.as<u32>(), m, k32.as<u32>());
  if (int rc = sort_pairs_u32(k32.as<u32>(), perm.as<u32>(), m, bit_count(nq), st, err))
    return rc;
  gather_final_kernel<<<blocks_for(m), 256, 0, st>>>(c.items.as<u64>(), c.dist.as<double>(), perm.as<u32>(), m, r.ids.as<u32>(), r.dist.as<double>());
  offsets_kernel<<<blocks_for(nq + 1), 256, 0, st>>>(k32.as<u32>(), m, nq, r.offsets.as<u64>());
  e = cudaStreamSynchronize(st);
  return cuda_status(e ? e : cudaGetLastError(), "finishing result");
}

// pairs (a << 32 | b) ascending: one "query" holding 2*m ids
static int finish_pairs(Collected& c, ResultState& r, cudaStream_t st)
{
  const u64 m = c.m;
  r.nq = 1;
  r.nids = 2 * m;
  r.hasDist = false;
  cudaError_t e;
  if ((e = result_alloc(r, sizeof(u64) * 2, sizeof(u32) * std::max<u64>(2 * m, 1), 0, st)))
    return cuda_status(e, "allocating result");
  u64 offs[2] = { 0, 2 * m };
  if ((e = cudaMemcpyAsync(r.offsets.p, offs, sizeof(offs), cudaMemcpyHostToDevice, st)))
    return cuda_status(e, "result offsets");
  if (m)
  {
    TmpBuf vals;
    if ((e = vals.ensure(sizeof(u32) * m, st)))
      return cuda_status(e, "allocating sort values");
    if (int rc = sort_pairs_u64(c.items.as<u64>(), vals.as<u32>(), m, 64, st, c.errp()))
      return rc;
    // (a << 32 | b) in little-endian memory is {b, a}: swap into {a, b}
    e = cudaMemcpyAsync(r.ids.p, c.items.p, sizeof(u64) * m, cudaMemcpyDeviceToDevice, st);
  }
  if (!e)
    e = cudaStreamSynchronize(st);
  return cuda_status(e, "finishing pairs");
}

__global__ void swap_pair_halves_kernel(u32* ids, u64 m)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
  {
    u32 lo = ids[2 * i], hi = ids[2 * i + 1];
    ids[2 * i] = hi;
    ids[2 * i + 1] = lo;
  }
}

// ---------------------------------------------------------------- host entry points
// stage a caller array in device memory
static int stage_input(TmpBuf& buf, const void* src, size_t bytes, int mem, cudaStream_t st, const void*& dptr)
{
  if (mem == OTG_MEM_DEVICE)
  {
    dptr = src;
    return OTG_OK;
  }
  if (cudaError_t e = buf.ensure(bytes, st))
    return cuda_status(e, "allocating query input");
  if (bytes)
    if (cudaError_t e = cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, st))
      return cuda_status(e, "copying query input");
  dptr = buf.p;
  return OTG_OK;
}

static int empty_result(u64 nq, ResultState& r, bool dist, cudaStream_t st)
{
  r.nq = nq;
  r.nids = 0;
  r.hasDist = dist;
  if (cudaError_t e = result_alloc(r, sizeof(u64) * (nq + 1), 4, dist ? 8 : 0, st))
    return cuda_status(e, "allocating result");
  cudaError_t e = cudaMemsetAsync(r.offsets.p, 0, sizeof(u64) * (nq + 1), st);
  if (!e)
    e = cudaStreamSynchronize(st);
  return cuda_status(e, "empty result");
}

// shapes of the batched query kernels: 0 = one query per thread; else warps per block (2, 4, 8) of
// the warp-per-query kernel | split code << 8 (no split, or the subtrees at depth 1, 2 or 3 become
// work items; otg_query.cuh). OTG_ALGO_DEFAULT lets the autotuner choose among all of them,
// OTG_ALGO_FILTERED among the warp shapes; the split depths offered depend on the batch size.
static std::vector<std::pair<int, const char*>> query_shapes(int algo, u64 nq)
{
  static const char* names[3][4] = { { "warp x2", "warp x2 split 1", "warp x2 split 2", "warp x2 split 3" },
                                     { "warp x4", "warp x4 split 1", "warp x4 split 2", "warp x4 split 3" },
                                     { "warp x8", "warp x8 split 1", "warp x8 split 2", "warp x8 split 3" } };
  std::vector<std::pair<int, const char*>> out;
  if (algo == OTG_ALGO_DEFAULT)
    out.push_back({ 0, "thread" });
  const u32 maxDepth = split_depth_limit(nq);
  const int warps[3] = { 2, 4, 8 };
  for (int w = 0; w < 3; ++w)
    for (u32 d = 0; d <= maxDepth; ++d)
      out.push_back({ warps[w] | int((d + 1) << 8), names[w][d] });
  return out;
}
// the shape used when the autotuner is off: 4 warps, the default split
constexpr int kDefaultQueryShape = 4;


template<typename T>
static int range_impl(const TreeState& t, const void* ranges, u64 nq, int mode, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                      const u32* qTree)
{
  TmpBuf in;
  const void* d;
  if (int rc = stage_input(in, ranges, sizeof(T) * 6 * nq, mem, st, d))
    return rc;
  if (t.n == 0 || nq == 0)
    return empty_result(nq, r, false, st);
  Collected c;
  auto tv = view<T>(t, qTree);
  T tl = tol_of<T>(tol);
  if (sizeof(T) == 8 && t.kind == OTG_KIND_POINTS && algo != OTG_ALGO_PLAIN_FP64)
  {
    // the batched kernel decides most node and point tests on FP32 images, the rest in FP64
    if (int rc = ensure_image32(const_cast<TreeState&>(t), st))
      return rc;
    tv.nodeImg = t.nodeBox32.as<float4>();
    tv.pointImg = t.geom32.as<float4>();
  }
  TmpBuf work;
  if (cudaError_t e = work.ensure(batch_work_bytes(nq), st))
    return cuda_status(e, "allocating the work counter");
  int launchRc = OTG_OK;
  int rc = collect(
    c, false, nq * 32,
    [&](Appender a, u32* err) {
      if (algo == OTG_ALGO_PLAIN_FP64)
        range_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), mode, tl, a, err);
      else
        launchRc = tune_run(query_key("range", algo, qTree, sizeof(T) == 8, t.kind, t.n, nq), query_shapes(algo, nq), kDefaultQueryShape, st, [&](int shape) {
          cudaMemsetAsync(a.count, 0, sizeof(unsigned long long), st);
          cudaMemsetAsync(err, 0, sizeof(u32), st);
          if (shape == 0)
          {
            range_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), mode, tl, a, err);
            return cuda_status(cudaGetLastError(), "launching the range search");
          }
          return batch_range<T>(tv, (const T*)d, u32(nq), mode, tl, a, work.as<u32>(), err, st, shape, work.bytes);
        });
    },
    st);
  if (launchRc)
    return launchRc;
  if (rc)
    return rc;
  r.filterTests = c.tests; // the FP32 pre-tests of the batched kernel and the ones left to FP64
  r.rechecks = c.rechecks;
  return finish_sorted_ids(c, nq, r, st, t.n);
}

template<typename T>
static int pick_impl(const TreeState& t, const void* pts, u64 nq, double tol, int algo, ResultState& r, int mem, cudaStream_t st, const u32* qTree)
{
  TmpBuf in;
  const void* d;
  if (int rc = stage_input(in, pts, sizeof(T) * 3 * nq, mem, st, d))
    return rc;
  if (t.n == 0 || nq == 0)
    return empty_result(nq, r, false, st);
  Collected c;
  auto tv = view<T>(t, qTree);
  T tl = tol_of<T>(tol);
  TmpBuf work;
  if (cudaError_t e = work.ensure(batch_work_bytes(nq), st))
    return cuda_status(e, "allocating the work counter");
  int launchRc = OTG_OK;
  int rc = collect(
    c, false, nq * 8,
    [&](Appender a, u32* err) {
      if (algo == OTG_ALGO_PLAIN_FP64)
        pick_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), tl, a, err);
      else
        launchRc = tune_run(query_key("pick", algo, qTree, sizeof(T) == 8, t.kind, t.n, nq), query_shapes(algo, nq), kDefaultQueryShape, st, [&](int shape) {
          cudaMemsetAsync(a.count, 0, sizeof(unsigned long long), st);
          cudaMemsetAsync(err, 0, sizeof(u32), st);
          if (shape == 0)
          {
            pick_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), tl, a, err);
            return cuda_status(cudaGetLastError(), "launching the pick search");
          }
          return batch_pick<T>(tv, (const T*)d, u32(nq), tl, a, work.as<u32>(), err, st, shape, work.bytes);
        });
    },
    st);
  if (launchRc)
    return launchRc;
  if (rc)
    return rc;
  return finish_sorted_ids(c, nq, r, st, t.n);
}

template<typename T>
static int frustum_impl(const TreeState& t, const void* planes, u64 np, u64 nq, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                        const u32* qTree)
{
  TmpBuf in;
  const void* d;
  if (int rc = stage_input(in, planes, sizeof(T) * 4 * np * nq, mem, st, d))
    return rc;
  if (t.n == 0 || nq == 0 || np == 0)
    return empty_result(nq, r, false, st);
  Collected c;
  auto tv = view<T>(t, qTree);
  T tl = tol_of<T>(tol);
  TmpBuf work;
  if (cudaError_t e = work.ensure(batch_work_bytes(nq), st))
    return cuda_status(e, "allocating the work counter");
  int launchRc = OTG_OK;
  int rc = collect(
    c, false, std::max<u64>(nq * 64, t.n / 4),
    [&](Appender a, u32* err) {
      if (algo == OTG_ALGO_PLAIN_FP64)
        frustum_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(np), u32(nq), tl, a, err);
      else
        launchRc = tune_run(query_key("frustum", algo, qTree, sizeof(T) == 8, t.kind, t.n, nq), query_shapes(algo, nq), kDefaultQueryShape, st, [&](int shape) {
          cudaMemsetAsync(a.count, 0, sizeof(unsigned long long), st);
          cudaMemsetAsync(err, 0, sizeof(u32), st);
          if (shape == 0)
          {
            frustum_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(np), u32(nq), tl, a, err);
            return cuda_status(cudaGetLastError(), "launching the frustum culling");
          }
          return batch_frustum<T>(tv, (const T*)d, u32(np), u32(nq), tl, a, work.as<u32>(), err, st, shape, work.bytes);
        });
    },
    st);
  if (launchRc)
    return launchRc;
  if (rc)
    return rc;
  return finish_sorted_ids(c, nq, r, st, t.n);
}

template<typename T>
static int plane_impl(const TreeState& t, const void* planes, u64 nq, bool positive, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                      const u32* qTree)
{
  TmpBuf in;
  const void* d;
  if (int rc = stage_input(in, planes, sizeof(T) * 4 * nq, mem, st, d))
    return rc;
  if (t.n == 0 || nq == 0)
    return empty_result(nq, r, false, st);
  Collected c;
  auto tv = view<T>(t, qTree);
  T tl = tol_of<T>(tol);
  TmpBuf work;
  if (cudaError_t e = work.ensure(batch_work_bytes(nq), st))
    return cuda_status(e, "allocating the work counter");
  int launchRc = OTG_OK;
  int rc = collect(
    c, false, std::max<u64>(nq * 64, positive ? t.n : t.n / 16),
    [&](Appender a, u32* err) {
      if (algo == OTG_ALGO_PLAIN_FP64)
        plane_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), positive ? 1 : 0, tl, a, err);
      else
        launchRc = tune_run(query_key(positive ? "plane positive" : "plane", algo, qTree, sizeof(T) == 8, t.kind, t.n, nq), query_shapes(algo, nq), kDefaultQueryShape, st,
                            [&](int shape) {
                              cudaMemsetAsync(a.count, 0, sizeof(unsigned long long), st);
                              cudaMemsetAsync(err, 0, sizeof(u32), st);
                              if (shape == 0)
                              {
                                plane_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), positive ? 1 : 0, tl, a, err);
                                return cuda_status(cudaGetLastError(), "launching the plane search");
                              }
                              return batch_plane<T>(tv, (const T*)d, u32(nq), positive, tl, a, work.as<u32>(), err, st, shape, work.bytes);
                            });
    },
    st);
  if (launchRc)
    return launchRc;
  if (rc)
    return rc;
  return finish_sorted_ids(c, nq, r, st, t.n);
}

// conditions given in host memory are checked here; device conditions are checked by the kernels
static int check_program_host(const QueryCond* conds, const u64* off, u64 nq, u64 nPlanes, u64 nBoxes)
{
  for (u64 q = 0; q < nq; ++q)
    if (off[q + 1] < off[q])
    {
      set_error("query offsets must not decrease");
      return OTG_ERR_INVALID_ARGUMENT;
    }
  for (u64 i = off[0]; i < off[nq]; ++i)
  {
    const QueryCond& c = conds[i];
    const bool ok = c.kind == kCondFrustum ? u64(c.first) + c.count <= nPlanes
                    : c.kind == kCondPlane ? c.first < nPlanes
                    : (c.kind == kCondRangeInside || c.kind == kCondRangeOverlap) ? c.first < nBoxes
                                                                                   : false;
    if (!ok)
    {
      set_error("query condition " + std::to_string(i) + ": unknown kind, or planes / box outside the given arrays");
      return OTG_ERR_INVALID_ARGUMENT;
    }
  }
  return OTG_OK;
}

template<typename T>
static int query_impl(const TreeState& t, const QueryCond* conds, const u64* off, u64 nq, const void* planes, const unsigned char* cross, u64 nPlanes,
                      const void* boxes, u64 nBoxes, int orOp, double tol, int algo, ResultState& r, int mem, cudaStream_t st)
{
  u64 nConds = 0;
  if (nq)
  {
    if (mem == OTG_MEM_HOST)
    {
      nConds = off[nq];
      if (int rc = check_program_host(conds, off, nq, nPlanes, nBoxes))
        return rc;
    }
    else
    {
      cudaError_t e = cudaMemcpyAsync(&nConds, off + nq, sizeof(u64), cudaMemcpyDeviceToHost, st);
      if (!e)
        e = cudaStreamSynchronize(st);
      if (e)
        return cuda_status(e, "reading the condition count");
    }
  }
  TmpBuf inC, inO, inP, inX, inB;
  const void *dC, *dO, *dP, *dX, *dB;
  if (int rc = stage_input(inC, conds, sizeof(QueryCond) * nConds, mem, st, dC))
    return rc;
  if (int rc = stage_input(inO, off, sizeof(u64) * (nq + 1), mem, st, dO))
    return rc;
  if (int rc = stage_input(inP, planes, sizeof(T) * 4 * nPlanes, mem, st, dP))
    return rc;
  if (int rc = stage_input(inX, cross, nPlanes, mem, st, dX))
    return rc;
  if (int rc = stage_input(inB, boxes, sizeof(T) * 6 * nBoxes, mem, st, dB))
    return rc;
  if (t.n == 0 || nq == 0)
    return empty_result(nq, r, false, st);
  QueryProgram<T> qp{ (const QueryCond*)dC, (const u64*)dO, (const T*)dP, (const unsigned char*)dX, (const T*)dB, nConds, nPlanes, nBoxes, orOp ? 1 : 0 };
  Collected c;
  auto tv = view<T>(t, nullptr);
  T tl = tol_of<T>(tol);
  TmpBuf work;
  if (cudaError_t e = work.ensure(batch_work_bytes(nq), st))
    return cuda_status(e, "allocating the work counter");
  int launchRc = OTG_OK;
  int rc = collect(
    c, false, std::max<u64>(nq * 64, t.n / 4),
    [&](Appender a, u32* err) {
      if (algo == OTG_ALGO_PLAIN_FP64)
        query_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, qp, u32(nq), tl, a, err);
      else
        launchRc = tune_run(query_key(orOp ? "query or" : "query and", algo, false, sizeof(T) == 8, t.kind, t.n, nq), query_shapes(algo, nq), kDefaultQueryShape, st,
                            [&](int shape) {
                              cudaMemsetAsync(a.count, 0, sizeof(unsigned long long), st);
                              cudaMemsetAsync(err, 0, sizeof(u32), st);
                              if (shape == 0)
                              {
                                query_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, qp, u32(nq), tl, a, err);
                                return cuda_status(cudaGetLastError(), "launching the combined query");
                              }
                              return batch_query_program<T>(tv, qp, u32(nq), tl, a, work.as<u32>(), err, st, shape, work.bytes);
                            });
    },
    st);
  if (launchRc)
    return launchRc;
  if (rc)
    return rc;
  return finish_sorted_ids(c, nq, r, st, t.n);
}

template<typename T>
static int knn_impl(const TreeState& t, const void* pts, u64 nq, const u32* k, u32 kAll, double maxDist, double tol, int algo, ResultState& r, int mem,
                    cudaStream_t st, const u32* qTree)
{
  TmpBuf in, kin, F;
  const void* d;
  const void* dk = nullptr;
  if (int rc = stage_input(in, pts, sizeof(T) * 3 * nq, mem, st, d))
    return rc;
  if (k)
    if (int rc = stage_input(kin, k, sizeof(u32) * nq, mem, st, dk))
      return rc;
  if (t.n == 0 || nq == 0)
    return empty_result(nq, r, true, st);
  if (algo != OTG_ALGO_PLAIN_FP64 && t.kind == OTG_KIND_POINTS && !qTree)
    return knn_filtered(const_cast<TreeState&>(t), d, (const u32*)dk, nq, kAll, maxDist, tol, r, st);
  if (cudaError_t e = F.ensure(sizeof(T) * nq, st))
    return cuda_status(e, "allocating kNN thresholds");
  auto tv = view<T>(t, qTree);
  T tl = tol_of<T>(tol);
  T F0 = maxDist < 0 ? Lim<T>::max() : upper_tol_host(T(maxDist), tl);
  // the heap bucket: the largest k of the batch (per-query k is reduced on the device)
  u32 kMax = kAll;
  if (dk)
  {
    TmpBuf m;
    cudaError_t e;
    if ((e = m.ensure(sizeof(u32), st)) || (e = cudaMemsetAsync(m.p, 0, sizeof(u32), st)))
      return cuda_status(e, "finding the largest k");
    max_u32_kernel<<<u32(std::min<u64>((nq + 255) / 256, 152 * 8)), 256, 0, st>>>((const u32*)dk, nq, m.as<u32>());
    if ((e = cudaMemcpyAsync(&kMax, m.p, sizeof(u32), cudaMemcpyDeviceToHost, st)) || (e = cudaStreamSynchronize(st)))
      return cuda_status(e, "finding the largest k");
  }
  const int bucket = knn_heap_bucket(kMax);
  Collected c;
  int rc = collect(
    c, true, nq * 16,
    [&](Appender a, u32* err) {
      launch_knn_threshold<T>(bucket, u32((nq + 127) / 128), st, tv, (const T*)d, u32(nq), (const u32*)dk, kAll, F0, tl, F.as<T>(), err);
      knn_collect_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), F.as<T>(), tl, a, err);
    },
    st);
  if (rc)
    return rc;
  return finish_by_distance(c, nq, t.n, r, st);
}

template<typename T>
static int ray_impl(const TreeState& t, const void* rays, u64 nq, double tol, double tolInc, double maxDist, bool first, int algo, ResultState& r,
                    int mem, cudaStream_t st, const u32* qTree)
{
  TmpBuf in, M;
  const void* d;
  if (int rc = stage_input(in, rays, sizeof(T) * 6 * nq, mem, st, d))
    return rc;
  if (t.n == 0 || nq == 0)
    return empty_result(nq, r, true, st);
  auto tv = view<T>(t, qTree);
  T tl = tol_of<T>(tol);
  T ti = T(tolInc);
  T md = maxDist < 0 ? Lim<T>::max() : T(maxDist);
  Collected c;
  int rc;
  if (!first)
  {
    TmpBuf work;
    if (cudaError_t e = work.ensure(batch_work_bytes(nq), st))
      return cuda_status(e, "allocating the work counter");
    int launchRc = OTG_OK;
    rc = collect(
      c, true, nq * 16,
      [&](Appender a, u32* err) {
        if (algo == OTG_ALGO_PLAIN_FP64)
          ray_all_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), tl, ti, md, a, err);
        else
          launchRc = tune_run(query_key("ray all", algo, qTree, sizeof(T) == 8, t.kind, t.n, nq), query_shapes(algo, nq), kDefaultQueryShape, st, [&](int shape) {
            cudaMemsetAsync(a.count, 0, sizeof(unsigned long long), st);
            cudaMemsetAsync(err, 0, sizeof(u32), st);
            if (shape == 0)
            {
              ray_all_plain_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), tl, ti, md, a, err);
              return cuda_status(cudaGetLastError(), "launching the ray query");
            }
            return batch_ray_all<T>(tv, (const T*)d, u32(nq), tl, ti, md, a, work.as<u32>(), err, st, shape, work.bytes);
          });
      },
      st);
    if (launchRc)
      return launchRc;
  }
  else
  {
    if (cudaError_t e = M.ensure(sizeof(T) * nq, st))
      return cuda_status(e, "allocating ray thresholds");
    rc = collect(
      c, true, nq * 4,
      [&](Appender a, u32* err) {
        ray_first_threshold_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), tl, ti, md, M.as<T>(), err);
        ray_first_collect_kernel<T><<<u32((nq + 127) / 128), 128, 0, st>>>(tv, (const T*)d, u32(nq), tl, ti, M.as<T>(), a, err);
      },
      st);
  }
  if (rc)
    return rc;
  return finish_by_distance(c, nq, t.n, r, st);
}

template<typename T>
static StructTree<T> struct_view(const TreeState& t)
{
  return StructTree<T>{ t.nodeBox.as<T>(),          t.ownerNode.as<u32>(), t.nodeParent.as<u32>(), t.nodeDepth.as<unsigned char>(),
                        t.sortedGeom.as<T>(),        t.sortedIds.as<u32>(), t.nodeLink.as<uint4>() };
}

template<typename T>
static int collide_impl(const TreeState& a, const TreeState& b, bool self, double tol, int algo, ResultState& r, cudaStream_t st)
{
  if (a.n == 0 || b.n == 0)
  {
    r.nq = 1;
    r.nids = 0;
    r.hasDist = false;
    if (cudaError_t e = result_alloc(r, sizeof(u64) * 2, 4, 0, st))
      return cuda_status(e, "allocating result");
    return cuda_status(cudaMemsetAsync(r.offsets.p, 0, sizeof(u64) * 2, st), "empty result");
  }
  Collected c;
  auto ta = view<T>(a), tb = view<T>(b);
  T tl = tol_of<T>(tol);
  const bool filtered = algo != OTG_ALGO_PLAIN_FP64;
  CollideSearch search;
  int searchRc = OTG_OK;
  int rc = collect(
    c, false, a.n * 4,
    [&](Appender ap, u32* err) {
      if (filtered)
        searchRc = collide_search_filtered(const_cast<TreeState&>(a), const_cast<TreeState&>(b), self, tol, ap, err, search, st);
      else
        collide_plain_kernel<T><<<u32((a.n + 127) / 128), 128, 0, st>>>(ta, tb, tl, self ? 1 : 0, ap, err);
    },
    st);
  if (searchRc)
    return searchRc;
  if (rc)
    return rc;
  u64 tests = 0, rechecks = 0;
  if (filtered && (rc = collide_search_stats(search, tests, rechecks, st)))
    return rc;
  const u64 m = c.m;
  TmpBuf keys, rej;
  cudaError_t e;
  if ((e = keys.ensure(sizeof(u64) * std::max<u64>(m, 1), st)) || (e = rej.ensure(sizeof(unsigned long long), st)))
    return cuda_status(e, "allocating pair filter");
  cudaMemsetAsync(rej.p, 0, sizeof(unsigned long long), st);
  if (m)
    collide_filter_kernel<T><<<blocks_for(m, 128), 128, 0, st>>>(struct_view<T>(a), struct_view<T>(b), self ? 1 : 0, c.items.as<u64>(), m, tl,
                                                                  keys.as<u64>(), rej.as<unsigned long long>());
  unsigned long long rejected = 0;
  e = cudaMemcpyAsync(&rejected, rej.p, sizeof(rejected), cudaMemcpyDeviceToHost, st);
  if (!e)
    e = cudaStreamSynchronize(st);
  if (e)
    return cuda_status(e, "filtering pairs");
  swap(c.items, keys);
  rc = finish_pairs(c, r, st); // rejected pairs carry key ~0 and sort last
  if (rc)
    return rc;
  const u64 kept = m - rejected;
  r.nids = 2 * kept;
  u64 offs[2] = { 0, 2 * kept };
  e = cudaMemcpyAsync(r.offsets.p, offs, sizeof(offs), cudaMemcpyHostToDevice, st);
  if (!e && kept)
    swap_pair_halves_kernel<<<blocks_for(kept), 256, 0, st>>>(r.ids.as<u32>(), kept);
  if (!e)
    e = cudaStreamSynchronize(st);
  r.filterTests = tests;
  r.rechecks = rechecks;
  return cuda_status(e, "finishing pairs");
}

int query_range(const TreeState& t, const void* ranges, u64 nq, int mode, double tol, int algo, ResultState& r, int mem, cudaStream_t st, const u32* qTree)
{
  return t.scalar == OTG_SCALAR_F64 ? range_impl<double>(t, ranges, nq, mode, tol, algo, r, mem, st, qTree)
                                    : range_impl<float>(t, ranges, nq, mode, tol, algo, r, mem, st, qTree);
}
int query_pick(const TreeState& t, const void* pts, u64 nq, double tol, int algo, ResultState& r, int mem, cudaStream_t st, const u32* qTree)
{
  return t.scalar == OTG_SCALAR_F64 ? pick_impl<double>(t, pts, nq, tol, algo, r, mem, st, qTree)
                                    : pick_impl<float>(t, pts, nq, tol, algo, r, mem, st, qTree);
}
int query_knn(const TreeState& t, const void* pts, u64 nq, const u32* k, u32 kAll, double maxDist, double tol, int algo, ResultState& r, int mem,
              cudaStream_t st, const u32* qTree)
{
  return t.scalar == OTG_SCALAR_F64 ? knn_impl<double>(t, pts, nq, k, kAll, maxDist, tol, algo, r, mem, st, qTree)
                                    : knn_impl<float>(t, pts, nq, k, kAll, maxDist, tol, algo, r, mem, st, qTree);
}
int query_combined(const TreeState& t, const void* conds, const u64* off, u64 nq, const void* planes, const unsigned char* cross, u64 nPlanes,
                   const void* boxes, u64 nBoxes, int orOp, double tol, int algo, ResultState& r, int mem, cudaStream_t st)
{
  const QueryCond* c = static_cast<const QueryCond*>(conds);
  return t.scalar == OTG_SCALAR_F64 ? query_impl<double>(t, c, off, nq, planes, cross, nPlanes, boxes, nBoxes, orOp, tol, algo, r, mem, st)
                                    : query_impl<float>(t, c, off, nq, planes, cross, nPlanes, boxes, nBoxes, orOp, tol, algo, r, mem, st);
}
int query_plane(const TreeState& t, const void* planes, u64 nq, bool positive, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                const u32* qTree)
{
  return t.scalar == OTG_SCALAR_F64 ? plane_impl<double>(t, planes, nq, positive, tol, algo, r, mem, st, qTree)
                                    : plane_impl<float>(t, planes, nq, positive, tol, algo, r, mem, st, qTree);
}
int query_frustum(const TreeState& t, const void* planes, u64 np, u64 nq, double tol, int algo, ResultState& r, int mem, cudaStream_t st,
                  const u32* qTree)
{
  return t.scalar == OTG_SCALAR_F64 ? frustum_impl<double>(t, planes, np, nq, tol, algo, r, mem, st, qTree)
                                    : frustum_impl<float>(t, planes, np, nq, tol, algo, r, mem, st, qTree);
}
int query_ray(const TreeState& t, const void* rays, u64 nq, double tol, double tolInc, double maxDist, bool first, int algo, ResultState& r, int mem,
              cudaStream_t st, const u32* qTree)
{
  return t.scalar == OTG_SCALAR_F64 ? ray_impl<double>(t, rays, nq, tol, tolInc, maxDist, first, algo, r, mem, st, qTree)
                                    : ray_impl<float>(t, rays, nq, tol, tolInc, maxDist, first, algo, r, mem, st, qTree);
}

// tree of each query of a forest: queries [qoff[t], qoff[t+1]) belong to tree t
__global__ void query_tree_kernel(const u64* __restrict__ qoff, u32 trees, u64 nq, u32* __restrict__ qTree)
{
  for (u64 q = blockIdx.x * u64(blockDim.x) + threadIdx.x; q < nq; q += u64(gridDim.x) * blockDim.x)
  {
    u32 lo = 0, hi = trees;
    while (hi - lo > 1)
    {
      const u32 m = (lo + hi) >> 1;
      if (qoff[m] <= q)
        lo = m;
      else
        hi = m;
    }
    qTree[q] = lo;
  }
}

int forest_query_trees(const TreeState& t, const u64* qoffHost, DevBuf& qoffDev, DevBuf& qTree, u64& nq, cudaStream_t st)
{
  const u32 trees = t.trees;
  if (!qoffHost || qoffHost[0] != 0)
  {
    set_error("query offsets must start at 0");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  for (u32 i = 0; i < trees; ++i)
    if (qoffHost[i + 1] < qoffHost[i])
    {
      set_error("query offsets must not decrease");
      return OTG_ERR_INVALID_ARGUMENT;
    }
  nq = qoffHost[trees];
  cudaError_t e;
  if ((e = qoffDev.ensure(sizeof(u64) * (trees + 1))) || (e = qTree.ensure(sizeof(u32) * std::max<u64>(nq, 1))))
    return cuda_status(e, "allocating query trees");
  if ((e = cudaMemcpyAsync(qoffDev.p, qoffHost, sizeof(u64) * (trees + 1), cudaMemcpyHostToDevice, st)))
    return cuda_status(e, "copying query offsets");
  if (nq)
    query_tree_kernel<<<blocks_for(nq), 256, 0, st>>>(qoffDev.as<u64>(), trees, nq, qTree.as<u32>());
  // the host offsets may be released by the caller once the copy has run
  if ((e = cudaStreamSynchronize(st)))
    return cuda_status(e, "mapping queries to trees");
  return OTG_OK;
}

int query_collide_self(const TreeState& t, double tol, int algo, ResultState& r, cudaStream_t st)
{
  return t.scalar == OTG_SCALAR_F64 ? collide_impl<double>(t, t, true, tol, algo, r, st) : collide_impl<float>(t, t, true, tol, algo, r, st);
}
int query_collide_pair(const TreeState& a, const TreeState& b, double tol, int algo, ResultState& r, cudaStream_t st)
{
  return a.scalar == OTG_SCALAR_F64 ? collide_impl<double>(a, b, false, tol, algo, r, st) : collide_impl<float>(a, b, false, tol, algo, r, st);
}

// ---------------------------------------------------------------- kNN without allocation
// Some callers cannot allocate device memory per call: a frame loop with a fixed memory budget
// (physics or game ticks that query neighbours every frame), code that must not trigger the
// implicit device synchronisation of cudaMalloc/cudaFree, or a pool-managed process that forbids
// allocations after start-up. For them the kNN query keeps its only scratch (the per-query
// threshold of the first pass and a status word) in a fixed array in the module's static device
// memory, and writes results straight into caller-owned per-query slots instead of a result
// object. The scratch is shared by every call on a device, so calls that overlap on the GPU
// (several host threads, or several streams) race on it and must be serialised by the caller.
constexpr u64 kNoAllocMaxQueries = u64(1) << 20;            // queries per call
constexpr u64 kNoAllocScratchBytes = 256 + 8 * kNoAllocMaxQueries; // status word, then one threshold per query
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noAllocScratch[kNoAllocScratchBytes];

// Pass 2 of the kNN query writing into slots: every entity with (min) distance < F is counted,
// and the smallest `cap` of them by (distance, id) are kept in the query's slot, in that order.
template<typename T>
__global__ void __launch_bounds__(128) knn_collect_slots_kernel(TreeView<T> tv, const T* __restrict__ pts, u32 nq, const T* __restrict__ Fin, T tol,
                                                                u32 cap, u32* __restrict__ counts, u32* __restrict__ ids, double* __restrict__ dist,
                                                                u32* err)
{
  using G = GeoD<T>;
  const u32 q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq)
    return;
  const T F = Fin[q];
  T p[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    p[c] = pts[u64(q) * 3 + c];
  u32* sid = ids + u64(q) * cap;
  double* sd = dist + u64(q) * cap;
  u32 found = 0, kept = 0;
  u32 stack[kStack];
  int sp = 0;
  u32 visits = 0;
  stack[sp++] = 0;
  while (sp > 0)
  {
    const u32 node = stack[--sp];
    const T* nb = tv.nodeBox + u64(node) * 6;
    if (G::wall_distance(p, nb, nb + 3) >= F)
      continue;
    const uint4 L = tv.link[node];
    if (L.z > tv.n || L.w > tv.n || L.y > L.z)
    {
      atomicOr(err, kErrStack);
      break;
    }
    for (u32 e = L.y; e < L.z; ++e)
    {
      const T d = entity_distance(tv, e, p, tol);
      if (!(d < F))
        continue;
      ++found;
      const double dd = double(d);
      const u32 id = tv.ids[e];
      // insertion into the sorted slot; the largest entry falls off a full slot
      u32 j = kept;
      while (j > 0 && (dd < sd[j - 1] || (dd == sd[j - 1] && id < sid[j - 1])))
      {
        if (j < cap)
        {
          sd[j] = sd[j - 1];
          sid[j] = sid[j - 1];
        }
        --j;
      }
      if (j < cap)
      {
        sd[j] = dd;
        sid[j] = id;
      }
      if (kept < cap)
        ++kept;
    }
    const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
    if (sp + int(cc) > kStack || (cc && u64(fc) + cc > tv.nNodes) || ++visits > tv.nNodes)
    {
      atomicOr(err, kErrStack);
      break;
    }
    for (u32 c = 0; c < cc; ++c)
      stack[sp++] = fc + c;
  }
  counts[q] = found;
}

// Device address of the static scratch on the current device, looked up once per device.
static int noalloc_scratch(unsigned char** out)
{
  static std::mutex lock;
  static unsigned char* addr[kNoAllocMaxDevices] = {};
  int dev = 0;
  if (cudaError_t e = cudaGetDevice(&dev))
    return cuda_status(e, "querying the current device");
  if (dev < 0 || dev >= kNoAllocMaxDevices)
  {
    set_error("device ordinal above the supported maximum of 63");
    return OTG_ERR_NOT_SUPPORTED;
  }
  std::lock_guard<std::mutex> g(lock);
  if (!addr[dev])
  {
    void* p = nullptr;
    if (cudaError_t e = cudaGetSymbolAddress(&p, g_noAllocScratch))
      return cuda_status(e, "looking up the no-allocation scratch");
    addr[dev] = (unsigned char*)p;
  }
  *out = addr[dev];
  return OTG_OK;
}

static bool device_accessible(const void* p)
{
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
  {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

template<typename T>
static int knn_noalloc_impl(const TreeState& t, const void* pts, u64 nq, u32 k, double maxDist, double tol, u32 cap, u32* counts, u32* ids,
                            double* dist, unsigned char* scratch, cudaStream_t st)
{
  cudaError_t e;
  if (t.n == 0)
  {
    e = cudaMemsetAsync(counts, 0, sizeof(u32) * nq, st);
    if (!e)
      e = cudaStreamSynchronize(st);
    return cuda_status(e, "empty kNN result");
  }
  u32* err = (u32*)scratch;
  T* F = (T*)(scratch + 256);
  if ((e = cudaMemsetAsync(err, 0, sizeof(u32), st)))
    return cuda_status(e, "clearing the kNN status");
  auto tv = view<T>(t);
  const T tl = tol_of<T>(tol);
  const T F0 = maxDist < 0 ? Lim<T>::max() : upper_tol_host(T(maxDist), tl);
  const u32 blocks = u32((nq + 127) / 128);
  launch_knn_threshold<T>(knn_heap_bucket(k), blocks, st, tv, (const T*)pts, u32(nq), nullptr, k, F0, tl, F, err);
  knn_collect_slots_kernel<T><<<blocks, 128, 0, st>>>(tv, (const T*)pts, u32(nq), F, tl, cap, counts, ids, dist, err);
  if ((e = cudaGetLastError()))
    return cuda_status(e, "launching the kNN query");
  u32 h = 0;
  e = cudaMemcpyAsync(&h, err, sizeof(u32), cudaMemcpyDeviceToHost, st);
  if (!e)
    e = cudaStreamSynchronize(st);
  if (e)
    return cuda_status(e, "running the kNN query");
  if (h & kErrStack)
  {
    set_error("traversal stack bound exceeded");
    return OTG_ERR_NOT_SUPPORTED;
  }
  return OTG_OK;
}

int query_knn_noalloc(const TreeState& t, const void* pts, u64 nq, u32 k, double maxDist, double tol, u32 cap, u32* counts, u32* ids, double* dist,
                      cudaStream_t st)
{
  unsigned char* scratch = nullptr;
  if (int rc = noalloc_scratch(&scratch)) // set-up happens even for n_queries == 0
    return rc;
  if (nq == 0)
    return OTG_OK;
  if (nq > kNoAllocMaxQueries)
  {
    set_error("n_queries above the no-allocation maximum of 1048576");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (k > u32(kKnnMaxK))
  {
    set_error("k above the supported maximum of 256");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (!pts || !counts || (cap && (!ids || !dist)))
  {
    set_error("points and counts (and ids and distances when slot_capacity > 0) must be given");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (!device_accessible(pts) || !device_accessible(counts) || (cap && (!device_accessible(ids) || !device_accessible(dist))))
  {
    set_error("points, counts, ids and distances must be device memory");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  return t.scalar == OTG_SCALAR_F64 ? knn_noalloc_impl<double>(t, pts, nq, k, maxDist, tol, cap, counts, ids, dist, scratch, st)
                                    : knn_noalloc_impl<float>(t, pts, nq, k, maxDist, tol, cap, counts, ids, dist, scratch, st);
}

} // namespace otg
