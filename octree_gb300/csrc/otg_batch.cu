// otg_batch.cu — batched RangeSearch, FrustumCulling, RayIntersectedAll, PlaneSearch and
// PlanePositiveSegmentation: persistent kernels in
// which each warp takes the next query from a shared counter (queries of uneven cost balance out,
// in one tree or across the trees of a forest) and answers it cooperatively:
//   * the node's own entities are tested by the 32 lanes in parallel (coalesced reads of the
//     tree-ordered geometry), hits compacted with a ballot into a per-warp shared buffer that is
//     flushed to the result with one atomic per flush;
//   * the node's children are tested by one lane each before they are pushed, so the depth-first
//     stack (in shared memory) only ever holds nodes the query enters.
// Every node and entity test is the reference predicate in the tree's scalar type, applied to the
// same nodes as the one-query-per-thread kernels of otg_query.cu, so the id sets are identical:
//   RangeSearch         core/ot_query.h:476-583
//   FrustumCulling      core/ot_query.h:767-833
//   RayIntersectedAll   core/ot_query.h:1928-2022
//   PlaneSearch         core/ot_query.h:612-636
//   PlanePositiveSegmentation core/ot_query.h:687-744
//   Query<And / Or>     core/ot_query.h:864-1026
//   PickSearch          core/ot_query.h:425-466
#include "otg_query.cuh"

namespace otg
{

constexpr u32 kItemBuf = 128;
constexpr u32 kContained = 1u << 31; // stack entry flag: the range contains the node (emit its subtree)
// Per-warp node stack. A step pops up to 32 nodes and pushes at most 8 children each, so it runs
// only while that cannot pass kWideStack - kWideReserve; beyond, one node per step (depth first)
// adds at most 7 entries per level over at most 19 levels.
constexpr int kWideStack = 768;
constexpr int kWideReserve = 160;

struct WarpSink
{
  u64* items;
  double* dist;
  u32 n;
};

// flushes the warp's buffered results to the appender (all lanes)
__device__ __forceinline__ void sink_flush(WarpSink& s, Appender& out, u32 lane)
{
  if (s.n == 0)
    return;
  unsigned long long base = 0;
  if (lane == 0)
    base = out.reserve(s.n);
  base = __shfl_sync(~0u, base, 0);
  for (u32 t = lane; t < s.n; t += 32)
    if (base + t < out.capacity)
    {
      out.items[base + t] = s.items[t];
      if (out.dist)
        out.dist[base + t] = s.dist[t];
    }
  __syncwarp();
  s.n = 0;
}

// appends the lanes with hit set (all lanes call)
__device__ __forceinline__ void sink_put(WarpSink& s, Appender& out, u32 lane, bool hit, u32 q, u32 id, double d)
{
  const u32 bal = __ballot_sync(~0u, hit);
  if (!bal)
    return;
  if (s.n + 32 > kItemBuf)
    sink_flush(s, out, lane);
  if (hit)
  {
    const u32 slot = s.n + __popc(bal & ((1u << lane) - 1));
    s.items[slot] = (u64(q) << 32) | id;
    if (out.dist)
      s.dist[slot] = d;
  }
  s.n += __popc(bal);
  __syncwarp();
}

// query kinds
constexpr int kRange = 0, kFrustum = 1, kRayAll = 2, kPlane = 3, kPlanePositive = 4, kQuery = 5, kPick = 6;

// ---- FP32 pre-tests of RangeSearch on FP64 point trees
// The FP64 tests (core/ot_query.h:476-583 with internal_geometry_module.h:190-252, :398-422):
//   node pruned  : some d with  maxL <= RN(nmin - tol)  or  maxR <= P        (overlap_by_min_point)
//   node inside  : every d with P <= nmin and maxR <= Q                      (range_contains_min_size)
//   point inside : every d with P < x < Q (tol != 0), or rmin <= x <= rmax (tol == 0)
// with P = RN(rmin - tol), Q = RN(rmax + tol), maxL = RN(rmin + RN(rmax - rmin)) per query and
// maxR = RN(nmin + nsize) per node. The images bound the FP64 values: a node's image holds
// lo = rd(nmin) and hi = ru(maxR), so nmin lies in [lo, succ(lo)) and maxR in (pred(hi), hi]; a
// point's image holds x32 = RN32(x), so x lies in (pred(x32), succ(x32)). Because floats are
// discrete, "succ(a) <= b" is "a < b" and "pred(a) >= b" is "a > b" for floats a, b, and each test
// below is decided where these bounds settle it, with per-query thresholds rounded down (lo) and up
// (hi) from the exact FP64 values:
//   P < x  : true if x32 > P.hi, false if x32 < P.lo      x < Q  : true if x32 < Q.lo, false if x32 > Q.hi
//   (the same for rmin <= x and x <= rmax with P = rmin, Q = rmax when tol == 0)
//   maxR <= P : true if hi <= P.lo, false if hi > P.hi   maxR <= Q : true if hi <= Q.lo, false if hi > Q.hi
//   P <= nmin : true if P.hi <= lo, false if lo < P.lo
//   maxL <= RN(nmin - tol) : true if ru(W + g) <= lo, false if lo < rd(W - g), W = RN(maxL + tol),
//     where the slack g = 2^-46 (M + tol) exceeds every FP64 rounding involved (M bounds the range's
//     and the root box's coordinates, so also every node's). RN is monotone, so maxL + tol <= nmin
//     gives maxL <= RN(nmin - tol); and nmin + g/2 < maxL + tol gives RN(nmin - tol) < maxL.
// Undecided tests run in FP64, so every answer is the FP64 answer.
struct RangeF32
{
  float w[3], s[3], plo[3], phi[3], qlo[3], qhi[3];
};

__device__ __forceinline__ void range_thresholds(const double* r, const double* rsize, const double* rootBox, double tol, RangeF32& f)
{
  double M = 0.0;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    M = fmax(M, fmax(fabs(r[d]), fabs(r[3 + d])));
    M = fmax(M, fmax(fabs(rootBox[d]), fabs(rootBox[d] + rootBox[3 + d])));
  }
  const double g = (M + fabs(tol)) * 0x1p-46;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    const double maxL = r[d] + rsize[d];
    const double P = r[d] - tol, Q = r[3 + d] + tol;
    const double W = maxL + tol;
    f.w[d] = __double2float_ru(W + g);
    f.s[d] = __double2float_rd(W - g);
    f.plo[d] = __double2float_rd(P);
    f.phi[d] = __double2float_ru(P);
    f.qlo[d] = __double2float_rd(Q);
    f.qhi[d] = __double2float_ru(Q);
  }
}

// The FP64 tests of the undecided cases, out of line: inlined, the compiler may evaluate them for
// every node and point beside the FP32 tests (predicated), which kept the FP64 pipe busy.
// the query's range as the caller passed it (6 doubles), and its size
__device__ __forceinline__ void range_load(const double* q, double r[6], double rsize[3])
{
#pragma unroll
  for (int c = 0; c < 6; ++c)
    r[c] = q[c];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    rsize[c] = r[3 + c] - r[c];
}
__device__ __noinline__ bool range_node_enters_fp64(const double* q, const double* nb, double tol)
{
  double r[6], rsize[3];
  range_load(q, r, rsize);
  return GeoD<double>::overlap_by_min_point(r, rsize, nb, nb + 3, tol);
}
__device__ __noinline__ bool range_node_inside_fp64(const double* q, const double* nb, double tol)
{
  double r[6], rsize[3];
  range_load(q, r, rsize);
  return GeoD<double>::range_contains_min_size(r, nb, nb + 3, tol);
}
__device__ __noinline__ bool range_point_inside_fp64(const double* q, const double* p, double tol)
{
  double r[6], rsize[3];
  range_load(q, r, rsize);
  return GeoD<double>::box_contains_point(r, p, tol);
}

// One query's FP64 setup, done beforehand by one thread per query (an FP64 instruction of a warp
// occupies this GPU's FP64 pipe for many cycles, so a warp doing one query's setup costs 32 times as
// much): the FP32 thresholds, and the flags of the root shortcut and of an empty range.
constexpr u32 kRangeAll = 1u, kRangeEmpty = 2u;
struct RangeQ
{
  RangeF32 f;
  u32 flags, pad;
};
static_assert(sizeof(RangeQ) == 80, "RangeQ: 20 words");

__global__ void __launch_bounds__(128) range_prepare_kernel(TreeView<double> tv, const double* __restrict__ ranges, u32 nq, double tol,
                                                            RangeQ* __restrict__ out)
{
  using G = GeoD<double>;
  for (u32 q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
  {
    const u32 root = query_root(tv, q);
    double r[6], rsize[3], rb[6];
    range_load(ranges + u64(q) * 6, r, rsize);
    const double* nb = tv.nodeBox + u64(root) * 6;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      rb[c] = nb[c];
      rb[3 + c] = nb[c] + nb[3 + c];
    }
    RangeQ o;
    o.flags = G::range_contains_box(r, rb, tol) ? kRangeAll : 0u; // root shortcut (:488-511)
    double vol = 1.0;                                             // zero-volume range -> empty (:514-519)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      vol *= rsize[c];
    if (vol <= 0.0)
      o.flags |= kRangeEmpty;
    range_thresholds(r, rsize, nb, tol, o.f);
    o.pad = 0;
    out[q] = o;
  }
}

// node: enter 0 (pruned) / 1 (entered) / 2 (undecided); inside 0 / 1 / 2 likewise
__device__ __forceinline__ void range_node_f32(const float4* __restrict__ img, u32 node, const RangeF32& f, int& enter, int& inside)
{
  const float4 mn = img[2 * size_t(node)], mx = img[2 * size_t(node) + 1];
  const float lo[3] = { mn.x, mn.y, mn.z }, hi[3] = { mx.x, mx.y, mx.z };
  bool anyPrune = false, allKeep = true, allIn = true, anyOut = false;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    anyPrune |= (f.w[d] <= lo[d]) | (hi[d] <= f.plo[d]);
    allKeep &= (lo[d] < f.s[d]) & (hi[d] > f.phi[d]);
    allIn &= (f.phi[d] <= lo[d]) & (hi[d] <= f.qlo[d]);
    anyOut |= (lo[d] < f.plo[d]) | (hi[d] > f.qhi[d]);
  }
  enter = anyPrune ? 0 : (allKeep ? 1 : 2);
  inside = anyOut ? 0 : (allIn ? 1 : 2);
}

// point: 0 outside, 1 inside, 2 undecided (also for a point without a finite image)
__device__ __forceinline__ int range_point_f32(const float4 p, const RangeF32& f)
{
  if (!(p.w < INFINITY))
    return 2;
  const float x[3] = { p.x, p.y, p.z };
  bool allIn = true, anyOut = false;
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    allIn &= (x[d] > f.phi[d]) & (x[d] < f.qlo[d]);
    anyOut |= (x[d] < f.plo[d]) | (x[d] > f.qhi[d]);
  }
  return anyOut ? 0 : (allIn ? 1 : 2);
}

template<typename T, int KIND>
struct BatchArgs
{
  TreeView<T> tv;
  const T* q;   // ranges (6 per query), planes (4 * np per query, 4 for the plane kinds), rays (6 per query) or points (3 per query)
  u32 np;       // planes per query
  u32 nq;
  int mode;     // RangeSearchMode
  T tol, tolInc, maxDist;
  Appender out;
  u32* work;          // counters (see batch_work_bytes), then the split items
  u32* err;
  QueryProgram<T> qp; // combined queries
  int phase;          // 0: whole queries; 1: top levels, deeper subtrees become items; 2: the items
  u32 splitCap;       // item capacity of the work buffer
  u32 splitDepth;     // depth of the subtrees that become items
  // range on FP64 point trees: one RangeQ per query (FP32 pre-tests); set only where out.count has
  // three slots (the item count, then the pre-tests and the undecided ones, added at the end)
  const void* prep = nullptr;
};

template<typename T, int KIND, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) batch_query_kernel(BatchArgs<T, KIND> a)
{
  static_assert(KIND >= kRange && KIND <= kPick, "every query kind has its own setup, node test and entity test below");
  using G = GeoD<T>;
  constexpr bool kRangeF32 = KIND == kRange && sizeof(T) == 8;
  __shared__ RangeF32 rangeF[kRangeF32 ? WARPS : 1];
  __shared__ u32 stackMem[WARPS][kWideStack];
  __shared__ u64 itemMem[WARPS][kItemBuf];
  __shared__ double distMem[KIND == kRayAll ? WARPS : 1][KIND == kRayAll ? kItemBuf : 1];
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  u32* stack = stackMem[w];
  WarpSink sink{ itemMem[w], KIND == kRayAll ? distMem[w] : nullptr, 0 };
  const TreeView<T>& tv = a.tv;
  u64* items = reinterpret_cast<u64*>(a.work + 4);
  u32 f32Tests = 0, f32Undecided = 0; // FP32 pre-tests of this lane (range on FP64 point trees)
  for (;;)
  {
    u32 q = 0, start = 0;
    if (a.phase == 2)
    {
      // the next (query, subtree) item left by the first phase
      u32 idx = 0;
      if (lane == 0)
        idx = atomicAdd(a.work + 1, 1u);
      idx = __shfl_sync(~0u, idx, 0);
      if (idx >= min(a.work[2], a.splitCap))
        break;
      const u64 item = items[idx];
      q = u32(item >> 32);
      start = u32(item);
      if (q >= a.nq)
        break;
    }
    else
    {
      if (lane == 0)
        q = atomicAdd(a.work, 1u);
      q = __shfl_sync(~0u, q, 0);
      if (q >= a.nq)
        break;
    }
    const u32 root = query_root(tv, q);
    const u32 idBase = id_base(tv, root);
    // ---- query setup (identical on all lanes)
    T r[6], rsize[3];
    const T* pl = nullptr;
    RayD<T> ray;
    bool skip = false;
    bool useF32 = false;
    if constexpr (kRangeF32)
    {
      if (a.prep)
      {
        // the query's prepared thresholds into the warp's shared copy, its flags to every lane
        const u32* src = reinterpret_cast<const u32*>(static_cast<const RangeQ*>(a.prep) + q);
        __syncwarp(); // the previous query's thresholds are read by every lane before they change
        if (lane < 18)
          reinterpret_cast<u32*>(&rangeF[w])[lane] = src[lane];
        const u32 flags = src[18];
        __syncwarp();
        useF32 = true;
        if (a.phase != 2 && (flags & kRangeAll))
        {
          const u32 nt = tv.qTree ? u32(tv.treeOff[root + 1] - tv.treeOff[root]) : tv.n;
          unsigned long long base = 0;
          if (lane == 0)
            base = a.out.reserve(nt);
          base = __shfl_sync(~0u, base, 0);
          for (u32 i = lane; i < nt; i += 32)
            if (base + i < a.out.capacity)
              a.out.items[base + i] = (u64(q) << 32) | i;
          continue;
        }
        skip = (flags & kRangeEmpty) != 0;
      }
    }
    if constexpr (KIND == kRange)
    {
      if (!useF32)
      {
      load_box(a.q + u64(q) * 6, r);
      if (a.phase != 2) // items continue queries that passed this setup in the first phase
      {
        T rb[6];
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
          rb[c] = tv.nodeBox[u64(root) * 6 + c];
          rb[3 + c] = tv.nodeBox[u64(root) * 6 + c] + tv.nodeBox[u64(root) * 6 + 3 + c];
        }
        if (G::range_contains_box(r, rb, a.tol)) // root shortcut (:488-511): every id of the tree
        {
          const u32 nt = tv.qTree ? u32(tv.treeOff[root + 1] - tv.treeOff[root]) : tv.n;
          unsigned long long base = 0;
          if (lane == 0)
            base = a.out.reserve(nt);
          base = __shfl_sync(~0u, base, 0);
          for (u32 i = lane; i < nt; i += 32)
            if (base + i < a.out.capacity)
              a.out.items[base + i] = (u64(q) << 32) | i;
          continue;
        }
      }
      T vol = T(1); // zero-volume range -> empty (:514-519)
#pragma unroll
      for (int c = 0; c < 3; ++c)
      {
        rsize[c] = T(r[3 + c] - r[c]);
        vol *= rsize[c];
      }
      skip = vol <= T(0);
      }
    }
    else if constexpr (KIND == kFrustum)
    {
      pl = a.q + u64(q) * a.np * 4;
      skip = a.np == 0;
    }
    else if constexpr (KIND == kPlane || KIND == kPlanePositive)
      pl = a.q + u64(q) * 4;
    else if constexpr (KIND == kPick)
    {
      pl = a.q + u64(q) * 3; // the point
      if (a.phase != 2)
      {
        T rb[6];
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
          rb[c] = tv.nodeBox[u64(root) * 6 + c];
          rb[3 + c] = tv.nodeBox[u64(root) * 6 + c] + tv.nodeBox[u64(root) * 6 + 3 + c];
        }
        skip = !G::box_contains_point(rb, pl, a.tol); // :430-431 the point outside the tree's box
      }
    }
    else if constexpr (KIND == kRayAll)
    {
      ray.make(a.q + u64(q) * 6, a.q + u64(q) * 6 + 3, a.tol, a.tolInc);
      skip = !ray.valid;
    }
    if (skip)
      continue;
    // ---- node test of one node (run by one lane per child)
    auto enters = [&](u32 node, bool& contained) -> bool {
      const T* nb = tv.nodeBox + u64(node) * 6;
      contained = false;
      if constexpr (KIND == kRange)
      {
        if constexpr (kRangeF32)
        {
          if (useF32)
          {
            int en, in;
            range_node_f32(tv.nodeImg, node, rangeF[w], en, in);
            ++f32Tests;
            f32Undecided += (en == 2 || (en != 0 && in == 2)) ? 1u : 0u;
            if (en == 0)
              return false;
            if (en == 2 && !range_node_enters_fp64(a.q + u64(q) * 6, nb, a.tol))
              return false;
            contained = in == 1;
            if (in == 2)
              contained = range_node_inside_fp64(a.q + u64(q) * 6, nb, a.tol);
            return true;
          }
          // FP64 trees without the pre-tests (box trees): the same tests, out of line, so that none of
          // their FP64 arithmetic is evaluated beside the FP32 path
          if (!range_node_enters_fp64(a.q + u64(q) * 6, nb, a.tol))
            return false;
          contained = range_node_inside_fp64(a.q + u64(q) * 6, nb, a.tol);
          return true;
        }
        T nmin[3] = { nb[0], nb[1], nb[2] }, nsize[3] = { nb[3], nb[4], nb[5] };
        if (!G::overlap_by_min_point(r, rsize, nmin, nsize, a.tol))
          return false;
        contained = G::range_contains_min_size(r, nmin, nsize, a.tol);
        return true;
      }
      else if constexpr (KIND == kFrustum)
      {
        for (u32 i = 0; i < a.np; ++i) // :779-795 first Hit selects, first Negative prunes
        {
          const int rel = G::box_plane(nb, nb + 3, pl[4 * i], pl + 4 * i + 1, a.tol);
          if (rel == 1)
            return true;
          if (rel == 0)
            return false;
        }
        return true;
      }
      else if constexpr (KIND == kPlane)
        return G::box_plane(nb, nb + 3, pl[0], pl + 1, a.tol) == 1; // :620-621 only nodes the plane hits
      else if constexpr (KIND == kPlanePositive)
      {
        const int rel = G::box_plane(nb, nb + 3, pl[0], pl + 1, a.tol); // :702-710 negative prunes, positive takes the subtree
        contained = rel == 2;
        return rel != 0;
      }
      else if constexpr (KIND == kQuery)
        return cond_combine(a.qp, q, a.err, [&](const QueryCond& c) { return cond_node(a.qp, c, nb, a.tol); });
      else if constexpr (KIND == kPick)
        return G::node_contains_point(nb, nb + 3, pl, a.tol);
      else if constexpr (KIND == kRayAll)
      {
        T en, ex;
        return ray.hit_node(nb, nb + 3, en, ex);
      }
    };
    u32 sp = 0;
    if (lane == 0)
    {
      bool contained;
      if (a.phase == 2)
      {
        stack[0] = start; // entered (its node test passed) in the first phase
        sp = 1;
      }
      else if (enters(root, contained))
      {
        stack[0] = root | (contained ? kContained : 0u);
        sp = 1;
      }
    }
    sp = __shfl_sync(~0u, sp, 0);
    __syncwarp();
    u32 visits = 0;
    bool bad = false;
    // the lane holding flat item f of a run of per-lane counts with inclusive prefix `incl`
    auto owner = [&](u32 incl, u32 f) -> u32 {
      u32 o = 0;
#pragma unroll
      for (u32 s = 16; s >= 1; s >>= 1)
        if (__shfl_sync(~0u, incl, o + s - 1) <= f)
          o += s;
      return o;
    };
    while (sp > 0)
    {
      // up to 32 nodes per step, one per lane; one at a time (depth first) near the stack's end. The
      // entities and children of the popped nodes are spread over the lanes as one flat run, so
      // consecutive lanes read consecutive entities of a node.
      const u32 take = (sp + 7u * 32u <= u32(kWideStack - kWideReserve)) ? min(sp, 32u) : 1u;
      sp -= take;
      const bool act = lane < take;
      const u32 entry = act ? stack[sp + lane] : 0u;
      __syncwarp();
      const u32 node = entry & ~kContained;
      uint4 L = make_uint4(0u, 0u, 0u, 0u);
      if (act)
        L = tv.link[node];
      visits += take;
      const bool badLane = act && (L.z > tv.n || L.w > tv.n || L.y > L.z || (L.x >> kChildShift) > 8u ||
                                   u64(L.x & kFirstChildMask) + (L.x >> kChildShift) > tv.nNodes);
      if (__any_sync(~0u, badLane) || visits > tv.nNodes)
      {
        bad = true;
        break;
      }
      bool whole = false;
      if constexpr (KIND == kRange || KIND == kPlanePositive)
      {
        whole = act && (entry & kContained);
        // whole subtrees without entity tests (range :549-567, positive side :711-726); a subtree is
        // one run of sortedIds
        u32 cm = __ballot_sync(~0u, whole);
        if (cm)
          sink_flush(sink, a.out, lane);
        while (cm)
        {
          const int src = __ffs(int(cm)) - 1;
          cm &= cm - 1;
          const u32 y = __shfl_sync(~0u, L.y, src), len = __shfl_sync(~0u, L.w, src) - y;
          unsigned long long base = 0;
          if (lane == 0)
            base = a.out.reserve(len);
          base = __shfl_sync(~0u, base, 0);
          for (u32 i = lane; i < len; i += 32)
            if (base + i < a.out.capacity)
              a.out.items[base + i] = (u64(q) << 32) | (tv.ids[y + i] - idBase);
        }
      }
      const bool tests = act && !whole;
      // entities of the popped nodes
      {
        const u32 cnt = tests ? L.z - L.y : 0u;
        u32 incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
          const u32 y = __shfl_up_sync(~0u, incl, o);
          if (lane >= u32(o))
            incl += y;
        }
        const u32 total = __shfl_sync(~0u, incl, 31);
        for (u32 f0 = 0; f0 < total; f0 += 32)
        {
          const u32 f = f0 + lane;
          const u32 o = owner(incl, min(f, total - 1));
          const u32 oy = __shfl_sync(~0u, L.y, o), oex = __shfl_sync(~0u, incl - cnt, o);
          const bool v = f < total;
          const u32 e = oy + (f - oex);
          bool hit = false;
          double d = 0.0;
          if (v)
          {
            if constexpr (KIND == kRange)
            {
              if (!tv.isBox)
              {
                int dec = 2;
                if constexpr (kRangeF32)
                  if (useF32)
                  {
                    dec = range_point_f32(tv.pointImg[e], rangeF[w]);
                    ++f32Tests;
                    f32Undecided += dec == 2 ? 1u : 0u;
                  }
                hit = dec == 1;
                if (dec == 2)
                {
                  if constexpr (kRangeF32)
                    hit = range_point_inside_fp64(a.q + u64(q) * 6, tv.geom + u64(e) * 3, a.tol);
                  else
                    hit = G::box_contains_point(r, tv.geom + u64(e) * 3, a.tol);
                }
              }
              else
              {
                T bx[6];
                load_box(tv.geom + u64(e) * 6, bx);
                hit = (a.mode == OTG_RANGE_OVERLAP) ? (G::box_relation(r, bx, a.tol) == -1) : G::contains_box_no_tol(r, bx);
              }
            }
            else if constexpr (KIND == kFrustum)
            {
              bool neg = false;
              for (u32 i = 0; i < a.np && !neg; ++i)
              {
                int rel;
                if (tv.isBox)
                {
                  const T* bx = tv.geom + u64(e) * 6;
                  T bsize[3] = { T(bx[3] - bx[0]), T(bx[4] - bx[1]), T(bx[5] - bx[2]) };
                  rel = G::box_plane(bx, bsize, pl[4 * i], pl + 4 * i + 1, a.tol);
                }
                else
                  rel = G::point_plane(tv.geom + u64(e) * 3, pl[4 * i], pl + 4 * i + 1, a.tol);
                neg = rel == 0;
              }
              hit = !neg;
            }
            else if constexpr (KIND == kPlane || KIND == kPlanePositive)
            {
              int rel; // ot_query.h:586-602 GetEntityPlaneRelation
              if (tv.isBox)
              {
                const T* bx = tv.geom + u64(e) * 6;
                T bsize[3] = { T(bx[3] - bx[0]), T(bx[4] - bx[1]), T(bx[5] - bx[2]) };
                rel = G::box_plane(bx, bsize, pl[0], pl + 1, a.tol);
              }
              else
                rel = G::point_plane(tv.geom + u64(e) * 3, pl[0], pl + 1, a.tol);
              hit = KIND == kPlane ? rel == 1 : rel != 0;
            }
            else if constexpr (KIND == kQuery)
            {
              const T* g = tv.geom + u64(e) * (tv.isBox ? 6 : 3);
              hit = cond_combine(a.qp, q, a.err, [&](const QueryCond& c) { return cond_entity(a.qp, c, g, tv.isBox != 0, a.tol); });
            }
            else if constexpr (KIND == kPick)
              hit = tv.isBox ? G::box_contains_point(tv.geom + u64(e) * 6, pl, a.tol) : G::points_equal(tv.geom + u64(e) * 3, pl, a.tol);
            else if constexpr (KIND == kRayAll)
            {
              T en, ex;
              hit = (tv.isBox ? ray.hit_box(tv.geom + u64(e) * 6, en, ex) : ray.hit_point(tv.geom + u64(e) * 3, en, ex)) &&
                    (a.maxDist == T(0) || en <= a.maxDist);
              d = double(en);
            }
          }
          sink_put(sink, a.out, lane, hit, q, hit ? tv.ids[e] - idBase : 0u, d);
        }
      }
      // children of the popped nodes, tested before they are pushed
      {
        const u32 cnt = tests ? (L.x >> kChildShift) : 0u;
        u32 incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
          const u32 y = __shfl_up_sync(~0u, incl, o);
          if (lane >= u32(o))
            incl += y;
        }
        const u32 total = __shfl_sync(~0u, incl, 31);
        for (u32 f0 = 0; f0 < total; f0 += 32)
        {
          const u32 f = f0 + lane;
          const u32 o = owner(incl, min(f, total - 1));
          const u32 ofc = __shfl_sync(~0u, L.x & kFirstChildMask, o), oex = __shfl_sync(~0u, incl - cnt, o);
          bool keep = false, contained = false;
          const u32 child = ofc + (f - oex);
          if (f < total)
            keep = enters(child, contained);
          if (a.phase == 1)
          {
            // subtrees at the split depth become items for any warp
            const bool defer = keep && tv.nodeDepth[child] >= a.splitDepth;
            const u32 dbal = __ballot_sync(~0u, defer);
            if (dbal)
            {
              u32 ibase = 0;
              if (lane == 0)
                ibase = atomicAdd(a.work + 2, u32(__popc(dbal)));
              ibase = __shfl_sync(~0u, ibase, 0);
              if (defer)
              {
                const u32 slot = ibase + __popc(dbal & ((1u << lane) - 1));
                if (slot < a.splitCap)
                  items[slot] = (u64(q) << 32) | child | (contained ? kContained : 0u);
                else
                  atomicOr(a.err, kErrStack);
              }
            }
            keep = keep && !defer;
          }
          const u32 bal = __ballot_sync(~0u, keep);
          if (sp + __popc(bal) > u32(kWideStack))
          {
            bad = true;
            break;
          }
          if (keep)
            stack[sp + __popc(bal & ((1u << lane) - 1))] = child | (contained ? kContained : 0u);
          sp += __popc(bal);
        }
      }
      __syncwarp();
      if (bad)
        break;
    }
    if (bad && lane == 0)
      atomicOr(a.err, kErrStack);
    sink_flush(sink, a.out, lane);
  }
  if constexpr (kRangeF32)
  {
    if (a.prep)
    {
      // the warp's counts, after the item count of the appender
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        f32Tests += __shfl_xor_sync(~0u, f32Tests, o);
        f32Undecided += __shfl_xor_sync(~0u, f32Undecided, o);
      }
      if (lane == 0)
      {
        atomicAdd(a.out.count + 1, (unsigned long long)f32Tests);
        atomicAdd(a.out.count + 2, (unsigned long long)f32Undecided);
      }
    }
  }
}

template<typename T, int KIND, int WARPS>
static int launch_batch_w(const BatchArgs<T, KIND>& a, cudaStream_t st)
{
  int dev = 0, sms = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (!e)
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!e)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, batch_query_kernel<T, KIND, WARPS>, WARPS * 32, 0);
  if (!e)
    e = cudaMemsetAsync(a.work, 0, 16, st);
  if (e)
    return cuda_status(e, "configuring the batched query kernel");
  const u64 resident = u64(sms) * std::max(per, 1);
  const u64 want = (u64(a.nq) + WARPS - 1) / WARPS;
  const u32 grid = u32(std::max<u64>(1, std::min<u64>(resident, want)));
  if (a.splitCap == 0)
  {
    batch_query_kernel<T, KIND, WARPS><<<grid, WARPS * 32, 0, st>>>(a);
    return cuda_status(cudaGetLastError(), "launching the batched query kernel");
  }
  // a small batch: the top levels of every query, then its subtrees spread over every resident warp
  BatchArgs<T, KIND> b = a;
  b.phase = 1;
  batch_query_kernel<T, KIND, WARPS><<<grid, WARPS * 32, 0, st>>>(b);
  b.phase = 2;
  batch_query_kernel<T, KIND, WARPS><<<u32(resident), WARPS * 32, 0, st>>>(b);
  return cuda_status(cudaGetLastError(), "launching the batched query kernel");
}

// shape: warps per block (2, 4 or 8) | split code << 8 (otg_query.cuh: shape_split_depth), autotuned
// workBytes: size of the work buffer; a batch is split only when the buffer holds its items
template<typename T, int KIND>
static int launch_batch(const BatchArgs<T, KIND>& a0, int shape, cudaStream_t st, size_t workBytes)
{
  if (workBytes < 16)
  {
    set_error("batched query work buffer below its 16 bytes of counters");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  BatchArgs<T, KIND> a = a0;
  a.phase = 0;
  a.splitDepth = shape_split_depth(shape, a.nq);
  const u64 items = a.splitDepth ? u64(a.nq) * split_items_per_query(a.splitDepth) : 0;
  a.splitCap = (items && a.tv.nodeDepth && workBytes >= 16 + sizeof(u64) * items) ? u32(items) : 0u;
  const int warps = shape & 0xff;
  if (warps == 2)
    return launch_batch_w<T, KIND, 2>(a, st);
  if (warps == 8)
    return launch_batch_w<T, KIND, 8>(a, st);
  return launch_batch_w<T, KIND, 4>(a, st);
}

template<typename T>
int batch_range(const TreeView<T>& tv, const T* ranges, u32 nq, int mode, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape, size_t workBytes)
{
  BatchArgs<T, kRange> a{ tv, ranges, 0, nq, mode, tol, T(0), T(0), out, work, err };
  TmpBuf prep;
  if constexpr (sizeof(T) == 8)
  {
    // FP64 point trees with FP32 images: the per-query setup by one thread per query
    if (tv.nodeImg && tv.pointImg && !tv.isBox && nq)
    {
      if (cudaError_t e = prep.ensure(sizeof(RangeQ) * nq, st))
        return cuda_status(e, "allocating the range setup");
      range_prepare_kernel<<<u32((nq + 127) / 128), 128, 0, st>>>(tv, ranges, nq, double(tol), prep.as<RangeQ>());
      a.prep = prep.p;
    }
  }
  return launch_batch<T, kRange>(a, shape, st, workBytes);
}
template<typename T>
int batch_frustum(const TreeView<T>& tv, const T* planes, u32 np, u32 nq, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape, size_t workBytes)
{
  return launch_batch<T, kFrustum>(BatchArgs<T, kFrustum>{ tv, planes, np, nq, 0, tol, T(0), T(0), out, work, err }, shape, st, workBytes);
}
template<typename T>
int batch_plane(const TreeView<T>& tv, const T* planes, u32 nq, bool positive, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape, size_t workBytes)
{
  if (positive)
    return launch_batch<T, kPlanePositive>(BatchArgs<T, kPlanePositive>{ tv, planes, 1, nq, 0, tol, T(0), T(0), out, work, err }, shape, st, workBytes);
  return launch_batch<T, kPlane>(BatchArgs<T, kPlane>{ tv, planes, 1, nq, 0, tol, T(0), T(0), out, work, err }, shape, st, workBytes);
}
template<typename T>
int batch_query_program(const TreeView<T>& tv, const QueryProgram<T>& qp, u32 nq, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape, size_t workBytes)
{
  BatchArgs<T, kQuery> a{ tv, nullptr, 0, nq, 0, tol, T(0), T(0), out, work, err };
  a.qp = qp;
  return launch_batch<T, kQuery>(a, shape, st, workBytes);
}
template<typename T>
int batch_pick(const TreeView<T>& tv, const T* pts, u32 nq, T tol, Appender out, u32* work, u32* err, cudaStream_t st, int shape, size_t workBytes)
{
  return launch_batch<T, kPick>(BatchArgs<T, kPick>{ tv, pts, 0, nq, 0, tol, T(0), T(0), out, work, err }, shape, st, workBytes);
}
template<typename T>
int batch_ray_all(const TreeView<T>& tv, const T* rays, u32 nq, T tol, T tolInc, T maxDist, Appender out, u32* work, u32* err, cudaStream_t st,
                  int shape, size_t workBytes)
{
  return launch_batch<T, kRayAll>(BatchArgs<T, kRayAll>{ tv, rays, 0, nq, 0, tol, tolInc, maxDist, out, work, err }, shape, st, workBytes);
}

template int batch_range<double>(const TreeView<double>&, const double*, u32, int, double, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_range<float>(const TreeView<float>&, const float*, u32, int, float, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_frustum<double>(const TreeView<double>&, const double*, u32, u32, double, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_frustum<float>(const TreeView<float>&, const float*, u32, u32, float, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_plane<double>(const TreeView<double>&, const double*, u32, bool, double, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_plane<float>(const TreeView<float>&, const float*, u32, bool, float, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_query_program<double>(const TreeView<double>&, const QueryProgram<double>&, u32, double, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_query_program<float>(const TreeView<float>&, const QueryProgram<float>&, u32, float, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_pick<double>(const TreeView<double>&, const double*, u32, double, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_pick<float>(const TreeView<float>&, const float*, u32, float, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_ray_all<double>(const TreeView<double>&, const double*, u32, double, double, double, Appender, u32*, u32*, cudaStream_t, int, size_t);
template int batch_ray_all<float>(const TreeView<float>&, const float*, u32, float, float, float, Appender, u32*, u32*, cudaStream_t, int, size_t);

} // namespace otg
