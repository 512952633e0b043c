// otg_knn.cu — batched GetNearestNeighbors for point trees: a persistent kernel with one warp per
// query (queries taken from a shared counter, so uneven k and uneven density balance out), an FP32
// outward-rounded distance filter, and an exact recheck of the few candidates near the k-th distance.
//
// Result semantics are those of the reference (core/ot_query.h:1208-1270 with AddEntityDistance
// :1058-1164): with F0 = U(maxDistance) (or the largest scalar when unbounded) and
// U(x) = fmax(tol, x * (1 + tol)) (GetValueWithToleranceUpper, :1033-1036), let S0 be the entities
// with distance d < F0. If |S0| >= k, F = U(d_k) with d_k the k-th smallest distance in S0; otherwise
// F = F0. The result is every entity with d < F, ordered by (d, id).
//
// Filter. Every entity gets FP32 bounds lo2 <= d^2 <= hi2 of the distance that the exact
// arithmetic computes: coordinates are stored as x32 = RN(x) with a per-entity error bound e, the
// query as a directed-rounding interval, and squares and sums use directed rounding; the bounds are
// then widened by a relative margin that covers the rounding of the exact formula itself. The warp
// keeps a shared-memory buffer of candidates with lo2 <= Fc2, where Fc is an FP32 upper bound of the
// final F derived from R2 = k-th smallest hi2 among entities certainly inside S0 (hi2 < F0^2).
// Because F <= U(d_k) <= U(sqrt(R2)) <= Fc, every result entity is a candidate. After the traversal
// only the candidates get the exact distance; they are sorted by (d, id) in shared memory and the
// reference rule is applied to them. Queries whose candidates do not fit the buffer (massive ties,
// or k above the buffer's limit) are answered by the plain one-thread-per-query kernels.
#include "otg_query.cuh"

#include <cfloat>
#include <cmath>
#include <cstddef>

namespace otg
{

constexpr float kInf = __builtin_huge_valf();

template<int CAP>
struct KnnWarpMem
{
  unsigned long long key[CAP]; // exact distance bits in the final sort
  u32 pos[CAP];                // sorted position of a candidate, then its entity id
  float lo2[CAP];
  float hi2[CAP];
  float tmp[CAP];
  u32 stackNode[kStack];
  float stackW[kStack];
};

struct KnnCounters
{
  unsigned long long out;      // result entries written
  unsigned long long tests;    // FP32 filter evaluations
  unsigned long long rechecks; // exact distance evaluations
  u32 work;                    // next query to take
  u32 fallbacks;
  u32 err;
  u32 pad;
};

template<typename T>
struct KnnArgs
{
  const uint4* link;
  const float4* nodeBox32; // 2 per node: {min rounded down, 0}, {max rounded up, 0}
  const float4* geom32;    // per sorted entity: {x, y, z, error bound}
  const T* geom;           // exact coordinates (sorted)
  const u32* ids;
  u32 n, nNodes;
  const T* pts;
  const u32* kArr;
  u32 kAll;
  u32 nq;
  const u32* order; // processing order of the queries (spatially sorted), or null
  T F0, tol;
  float F0hi, F0lo2, tolHi, onePlusTolHi, widenLo, widenHi;
  u32 kLimit;
  KnnCounters* ctr;
  u32* fallback;
  u64* start;
  u32* count;
  u32* outIds;
  double* outDist;
  u64 outCap;
};

// ---------------------------------------------------------------- FP32 images
// point: {x, y, z, e} with x = RN(x64) and e >= max |x64 - x| inflated by 2^-20 relative (the
// per-entity bound arithmetic below relies on that margin); e = +inf and x = 0 for coordinates
// outside the FP32 range (such entities always pass the filter).
template<typename T>
__global__ void point_image_kernel(const T* __restrict__ geom, u64 n, float4* __restrict__ out)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    float v[3];
    double e = 0.0;
    bool ok = true;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      const double x = double(geom[i * 3 + c]);
      const float f = __double2float_rn(x);
      ok &= isfinite(f);
      v[c] = f;
      e = fmax(e, fabs(x - double(f)));
    }
    out[i] = ok ? make_float4(v[0], v[1], v[2], __fmul_ru(__double2float_ru(e), 1.f + 0x1p-20f)) : make_float4(0.f, 0.f, 0.f, kInf);
  }
}

// Node boxes rounded outward: MinPoint geometry {min, size} (max = min + size), or the exact MBR max.
template<typename T>
__global__ void node_image_kernel(const T* __restrict__ nodeBox, const T* __restrict__ nodeMax, u64 m, float4* __restrict__ out)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
  {
    float lo[3], hi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      const double mn = double(nodeBox[i * 6 + c]);
      const double mx = nodeMax ? double(nodeMax[i * 3 + c]) : mn + double(nodeBox[i * 6 + 3 + c]);
      lo[c] = __double2float_rd(mn);
      hi[c] = __double2float_ru(mx);
    }
    out[2 * i] = make_float4(lo[0], lo[1], lo[2], 0.f);
    out[2 * i + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
  }
}

// ---------------------------------------------------------------- device helpers
// The per-node and per-entity bounds use round-to-nearest FP32 only (directed-rounding FP32
// instructions are much slower on this GPU); every rounding is covered by an explicit margin.
// With u = 2^-24, a round-to-nearest result r of a normal operation is within u|r| of the exact
// value, and sums and products of non-negative values gain at most a factor (1 + u) each.

// lower bound of the squared distance from the query interval [plo, phi] to an outward-rounded
// node box: each positive gap is shrunk by 2^-22 relative (covers its own rounding), the sum of
// squares by 2^-20 (covers four roundings), then by the caller's margin.
__device__ __forceinline__ float node_w2(const float4* __restrict__ nb, u32 node, const float* plo, const float* phi, float widenLo)
{
  const float4 mn = nb[2 * size_t(node)], mx = nb[2 * size_t(node) + 1];
  const float a[3] = { mn.x, mn.y, mn.z }, b[3] = { mx.x, mx.y, mx.z };
  float w2 = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c)
  {
    const float g = fmaxf(fmaxf(a[c] - phi[c], plo[c] - b[c]), 0.f) * (1.f - 0x1p-22f);
    w2 = fmaf(g, g, w2);
  }
  return w2 * ((1.f - 0x1p-20f) * widenLo);
}

// Bounds lo2 <= d^2 <= hi2 of the squared distance between the query (p32 = RN(p), per-coordinate
// error at most Sq, inflated by 2^-20) and an entity image {x32, e} (e inflated by 2^-20):
//   t = RN(x32 - p32) is within u|t| + e + Sq of the exact difference;
//   E = RN(|t| 2^-20 + RN(e + Sq)) >= 15u|t| + (e + Sq)_exact (1 + 12u) covers that error and the
//   rounding of |t| + E and |t| - E; the sums of squares are then widened by the caller's
//   margins, which also cover the rounding of the exact distance formula.
__device__ __forceinline__ void entity_bounds(float4 g, const float* p32, float Sq, float widenLo, float widenHi, float& l2, float& h2)
{
  const float x[3] = { g.x, g.y, g.z };
  const float S = g.w + Sq;
  float L = 0.f, H = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c)
  {
    const float a = fabsf(x[c] - p32[c]);
    const float E = fmaf(a, 0x1p-20f, S);
    const float hi = a + E;
    const float lo = fmaxf(a - E, 0.f);
    L = fmaf(lo, lo, L);
    H = fmaf(hi, hi, H);
  }
  l2 = fmaxf(fmaf(L, widenLo, -0x1p-140f), 0.f);
  h2 = fmaf(H, widenHi, 0x1p-140f);
}

__device__ __forceinline__ u32 pow2_at_least32(u32 v)
{
  return v <= 32 ? 32u : 1u << (32 - __clz(v - 1));
}

// ascending bitonic sort of n2 (a power of two) floats by one warp
__device__ __forceinline__ void warp_sort_f32(float* v, u32 n2, u32 lane)
{
  for (u32 size = 2; size <= n2; size <<= 1)
    for (u32 stride = size >> 1; stride > 0; stride >>= 1)
    {
      for (u32 t = lane; t < n2 / 2; t += 32)
      {
        const u32 i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
        const u32 j = i + stride;
        const bool up = (i & size) == 0;
        const float x = v[i], y = v[j];
        if ((x > y) == up && x != y)
        {
          v[i] = y;
          v[j] = x;
        }
      }
      __syncwarp();
    }
}

// ascending bitonic sort of (key, value) pairs by (key, value)
__device__ __forceinline__ void warp_sort_pairs(unsigned long long* k, u32* v, u32 n2, u32 lane)
{
  for (u32 size = 2; size <= n2; size <<= 1)
    for (u32 stride = size >> 1; stride > 0; stride >>= 1)
    {
      for (u32 t = lane; t < n2 / 2; t += 32)
      {
        const u32 i = ((t & ~(stride - 1)) << 1) | (t & (stride - 1));
        const u32 j = i + stride;
        const bool up = (i & size) == 0;
        const unsigned long long ki = k[i], kj = k[j];
        const u32 vi = v[i], vj = v[j];
        const bool greater = ki > kj || (ki == kj && vi > vj);
        const bool differ = ki != kj || vi != vj;
        if (differ && greater == up)
        {
          k[i] = kj;
          k[j] = ki;
          v[i] = vj;
          v[j] = vi;
        }
      }
      __syncwarp();
    }
}

// Recomputes the candidate bound from the buffer and drops candidates above it.
template<typename T, int CAP>
__device__ __forceinline__ void knn_flush(KnnWarpMem<CAP>& W, const KnnArgs<T>& a, u32 k, u32 lane, u32& bufN, float& Fc2)
{
  __syncwarp();
  const u32 n2 = pow2_at_least32(bufN);
  for (u32 i = lane; i < n2; i += 32)
    W.tmp[i] = (i < bufN && W.hi2[i] < a.F0lo2) ? W.hi2[i] : kInf;
  __syncwarp();
  warp_sort_f32(W.tmp, n2, lane);
  // round-to-nearest with a 2^-20 margin per step keeps every value an upper bound
  const float R2 = k <= n2 ? W.tmp[k - 1] : kInf;
  const float Rhi = sqrtf(R2) * (1.f + 0x1p-20f);
  const float Fc = fmaxf(a.tolHi, fminf(Rhi, a.F0hi) * a.onePlusTolHi);
  const float nFc2 = (Fc * Fc) * (1.f + 0x1p-20f);
  Fc2 = fminf(Fc2, nFc2);
  const u32 lt = (1u << lane) - 1;
  u32 kept = 0;
  for (u32 base = 0; base < bufN; base += 32)
  {
    const u32 i = base + lane;
    bool keep = false;
    u32 pp = 0;
    float l = 0.f, h = 0.f;
    if (i < bufN)
    {
      pp = W.pos[i];
      l = W.lo2[i];
      h = W.hi2[i];
      keep = l <= Fc2;
    }
    const u32 bal = __ballot_sync(~0u, keep);
    __syncwarp();
    if (keep)
    {
      const u32 s = kept + __popc(bal & lt);
      W.pos[s] = pp;
      W.lo2[s] = l;
      W.hi2[s] = h;
    }
    kept += __popc(bal);
    __syncwarp();
  }
  bufN = kept;
}

template<typename T, int CAP, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) knn_filtered_kernel(KnnArgs<T> a)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const u32 lane = threadIdx.x & 31;
  KnnWarpMem<CAP>& W = reinterpret_cast<KnnWarpMem<CAP>*>(smem)[threadIdx.x >> 5];
  const u32 lt = (1u << lane) - 1;
  unsigned long long tests = 0, rechecks = 0;
  for (;;)
  {
    u32 item = 0;
    if (lane == 0)
      item = atomicAdd(&a.ctr->work, 1u);
    item = __shfl_sync(~0u, item, 0);
    if (item >= a.nq)
      break;
    const u32 q = a.order ? a.order[item] : item;
    const u32 k = a.kArr ? a.kArr[q] : a.kAll;
    if (k == 0) // ot_query.h:1217-1219: no neighbour requested -> empty result
    {
      if (lane == 0)
        a.count[q] = 0;
      continue;
    }
    if (k > a.kLimit)
    {
      if (lane == 0)
      {
        a.fallback[atomicAdd(&a.ctr->fallbacks, 1u)] = q;
        a.count[q] = 0;
      }
      continue;
    }
    // query: p32 = RN(p) with |p - p32| <= 2^-24 |p32| + 2^-150 <= Sq / 2 (doubled margin);
    // [plo, phi] = p32 -/+ 2 Sq encloses p after its own rounding
    T p[3];
    float plo[3], phi[3], p32[3];
    float ap = 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      p[c] = a.pts[u64(q) * 3 + c];
      p32[c] = float(p[c]);
      ap = fmaxf(ap, fabsf(p32[c]));
    }
    float Sq = sizeof(T) == 4 ? 0.f : fmaf(ap, 0x1p-23f, 0x1p-140f);
    if (!(ap < kInf))
    {
      // a query outside the FP32 range: every entity is a candidate
      p32[0] = p32[1] = p32[2] = 0.f;
      Sq = kInf;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      plo[c] = p32[c] - 2.f * Sq;
      phi[c] = p32[c] + 2.f * Sq;
    }
    u32 bufN = 0;
    float Fc2;
    {
      const float Fc = fmaxf(a.tolHi, a.F0hi * a.onePlusTolHi);
      Fc2 = (Fc * Fc) * (1.f + 0x1p-20f);
    }
    u32 flushAt = min(u32(CAP), max(64u, 2 * k + 32));
    bool overflow = false;
    int sp = 1;
    if (lane == 0)
    {
      W.stackNode[0] = 0;
      W.stackW[0] = node_w2(a.nodeBox32, 0, plo, phi, a.widenLo);
    }
    __syncwarp();
    u32 visits = 0;
    while (sp > 0)
    {
      --sp;
      const u32 node = W.stackNode[sp];
      const float w2 = W.stackW[sp];
      __syncwarp();
      if (w2 > Fc2)
        continue;
      if (++visits > a.nNodes)
      {
        overflow = true;
        break;
      }
      const uint4 L = a.link[node];
      if (L.z > a.n || L.y > L.z)
      {
        overflow = true;
        break;
      }
      for (u32 base = L.y; base < L.z; base += 32)
      {
        if (bufN + 32 > flushAt)
        {
          knn_flush<T, CAP>(W, a, k, lane, bufN, Fc2);
          if (bufN + 32 > flushAt)
          {
            flushAt = CAP;
            if (bufN + 32 > flushAt)
            {
              overflow = true;
              break;
            }
          }
        }
        const u32 e = base + lane;
        float l2 = kInf, h2 = kInf;
        bool keep = false;
        if (e < L.z)
        {
          entity_bounds(a.geom32[e], p32, Sq, a.widenLo, a.widenHi, l2, h2);
          keep = l2 <= Fc2;
        }
        const u32 bal = __ballot_sync(~0u, keep);
        if (keep)
        {
          const u32 s = bufN + __popc(bal & lt);
          W.pos[s] = e;
          W.lo2[s] = l2;
          W.hi2[s] = h2;
        }
        bufN += __popc(bal);
        tests += min(32u, L.z - base);
      }
      if (overflow)
        break;
      const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
      if (cc)
      {
        if (u64(fc) + cc > a.nNodes || sp + int(cc) > kStack)
        {
          overflow = true;
          break;
        }
        float cw = kInf;
        bool ok = false;
        if (lane < cc)
        {
          cw = node_w2(a.nodeBox32, fc + lane, plo, phi, a.widenLo);
          ok = cw <= Fc2;
        }
        const u32 bal = __ballot_sync(~0u, ok);
        u32 rank = 0;
        for (u32 j = 0; j < cc; ++j)
        {
          const float wj = __shfl_sync(~0u, cw, j);
          if (((bal >> j) & 1u) && (wj > cw || (wj == cw && j > lane)))
            ++rank;
        }
        if (ok)
        {
          W.stackNode[sp + rank] = fc + lane;
          W.stackW[sp + rank] = cw;
        }
        sp += __popc(bal);
        __syncwarp();
      }
    }
    if (!overflow)
      knn_flush<T, CAP>(W, a, k, lane, bufN, Fc2);
    if (overflow)
    {
      if (lane == 0)
      {
        a.fallback[atomicAdd(&a.ctr->fallbacks, 1u)] = q;
        a.count[q] = 0;
      }
      __syncwarp();
      continue;
    }
    // exact distances of the candidates, then (distance, id) order
    for (u32 i = lane; i < bufN; i += 32)
    {
      const u32 e = W.pos[i];
      const T d = GeoD<T>::distance(p, a.geom + u64(e) * 3);
      W.key[i] = (unsigned long long)__double_as_longlong(double(d));
      W.pos[i] = a.ids[e];
    }
    const u32 n2 = pow2_at_least32(bufN);
    for (u32 i = bufN + lane; i < n2; i += 32)
    {
      W.key[i] = ~0ull;
      W.pos[i] = ~0u;
    }
    __syncwarp();
    warp_sort_pairs(W.key, W.pos, n2, lane);
    rechecks += bufN;
    // distances are non-negative: comparing bit patterns as integers orders them like values
    const unsigned long long F0bits = (unsigned long long)__double_as_longlong(double(a.F0));
    u32 below0 = 0;
    for (u32 base = 0; base < bufN; base += 32)
    {
      const u32 i = base + lane;
      below0 += __popc(__ballot_sync(~0u, i < bufN && W.key[i] < F0bits));
    }
    const T F = below0 >= k ? upper_tol(T(__longlong_as_double((long long)W.key[k - 1])), a.tol) : a.F0;
    const unsigned long long Fbits = (unsigned long long)__double_as_longlong(double(F));
    u32 m = 0;
    for (u32 base = 0; base < bufN; base += 32)
    {
      const u32 i = base + lane;
      m += __popc(__ballot_sync(~0u, i < bufN && W.key[i] < Fbits));
    }
    unsigned long long s0 = 0;
    if (lane == 0)
      s0 = atomicAdd(&a.ctr->out, (unsigned long long)m);
    s0 = __shfl_sync(~0u, s0, 0);
    if (s0 + m <= a.outCap)
      for (u32 i = lane; i < m; i += 32)
      {
        a.outIds[s0 + i] = W.pos[i];
        a.outDist[s0 + i] = __longlong_as_double((long long)W.key[i]);
      }
    if (lane == 0)
    {
      a.start[q] = s0;
      a.count[q] = m;
    }
    __syncwarp();
  }
  if (lane == 0)
  {
    atomicAdd(&a.ctr->tests, tests);
    atomicAdd(&a.ctr->rechecks, rechecks);
  }
}

// ---------------------------------------------------------------- query order, k statistics
// Morton order of the query points in the tree's space (10 bits per dimension): neighbouring
// queries then walk the same nodes, which keeps the traversal in L2.
__global__ void iota_order_kernel(u32* __restrict__ order, u64 nq)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < nq; i += u64(gridDim.x) * blockDim.x)
    order[i] = u32(i);
}

template<typename T>
__global__ void query_key_kernel(const T* __restrict__ pts, u64 nq, const Space<T>* __restrict__ sp, u32* __restrict__ keys, u32* __restrict__ idx)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < nq; i += u64(gridDim.x) * blockDim.x)
  {
    u32 c[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
      const float ext = float(sp->max[d] - sp->min[d]);
      const float rel = ext > 0.f ? float(pts[i * 3 + d] - sp->min[d]) / ext : 0.f;
      const float v = rel * 1024.f;
      c[d] = v <= 0.f ? 0u : (v >= 1023.f ? 1023u : u32(v));
    }
    keys[i] = u32(encode3(c[0], c[1], c[2]));
    idx[i] = u32(i);
  }
}

__global__ void k_stats_kernel(const u32* __restrict__ k, u64 nq, u32* __restrict__ kmax, unsigned long long* __restrict__ ksum)
{
  u32 mx = 0;
  unsigned long long s = 0;
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < nq; i += u64(gridDim.x) * blockDim.x)
  {
    mx = max(mx, k[i]);
    s += k[i];
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    mx = max(mx, __shfl_xor_sync(~0u, mx, o));
    s += __shfl_xor_sync(~0u, s, o);
  }
  if ((threadIdx.x & 31) == 0)
  {
    atomicMax(kmax, mx);
    atomicAdd(ksum, s);
  }
}

// ---------------------------------------------------------------- CSR assembly
constexpr u32 kFromFallback = 1u << 31; // high bit of start (as u64 bit 63): the entry lives in the plain result

__global__ void fallback_points_kernel(const u32* __restrict__ fb, u32 nfb, const void* __restrict__ pts, u32 ptBytes, const u32* __restrict__ kArr,
                                       u32 kAll, unsigned char* __restrict__ outPts, u32* __restrict__ outK)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < nfb; i += gridDim.x * blockDim.x)
  {
    const u32 q = fb[i];
    const unsigned char* src = static_cast<const unsigned char*>(pts) + u64(q) * ptBytes;
    for (u32 b = 0; b < ptBytes; ++b)
      outPts[u64(i) * ptBytes + b] = src[b];
    outK[i] = kArr ? kArr[q] : kAll;
  }
}

__global__ void fallback_slots_kernel(const u32* __restrict__ fb, u32 nfb, const u64* __restrict__ off, u64* __restrict__ start, u32* __restrict__ count)
{
  for (u32 i = blockIdx.x * blockDim.x + threadIdx.x; i < nfb; i += gridDim.x * blockDim.x)
  {
    const u32 q = fb[i];
    start[q] = off[i] | (u64(kFromFallback) << 32);
    count[q] = u32(off[i + 1] - off[i]);
  }
}


__device__ __forceinline__ u64 block_scan_u64(u64 v, u64* warpSums, u64& total)
{
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  u64 x = v;
  for (int o = 1; o < 32; o <<= 1)
  {
    const u64 y = __shfl_up_sync(~0u, x, o);
    if (lane >= u32(o))
      x += y;
  }
  if (lane == 31)
    warpSums[w] = x;
  __syncthreads();
  if (w == 0)
  {
    u64 s = lane < kScanThreads / 32 ? warpSums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1)
    {
      const u64 y = __shfl_up_sync(~0u, s, o);
      if (lane >= u32(o))
        s += y;
    }
    if (lane < kScanThreads / 32)
      warpSums[lane] = s;
  }
  __syncthreads();
  total = warpSums[kScanThreads / 32 - 1];
  const u64 before = w ? warpSums[w - 1] : 0;
  __syncthreads();
  return before + x - v; // exclusive
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const u32* __restrict__ cnt, u64 n, u64* __restrict__ tileSums)
{
  __shared__ u64 ws[kScanThreads / 32];
  const u64 base = u64(blockIdx.x) * kScanTile + u64(threadIdx.x) * kScanItems;
  u64 s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
    if (base + j < n)
      s += cnt[base + j];
  u64 total;
  block_scan_u64(s, ws, total);
  if (threadIdx.x == 0)
    tileSums[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place; tileSums[tiles] = grand total
__global__ void __launch_bounds__(kScanThreads) scan_tiles_kernel(u64* __restrict__ tileSums, u64 tiles)
{
  __shared__ u64 ws[kScanThreads / 32];
  u64 carry = 0;
  for (u64 base = 0; base < tiles; base += kScanThreads)
  {
    const u64 i = base + threadIdx.x;
    const u64 v = i < tiles ? tileSums[i] : 0;
    u64 total;
    const u64 ex = block_scan_u64(v, ws, total);
    if (i < tiles)
      tileSums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0)
    tileSums[tiles] = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const u32* __restrict__ cnt, u64 n, const u64* __restrict__ tileSums, u64* __restrict__ off)
{
  __shared__ u64 ws[kScanThreads / 32];
  const u64 base = u64(blockIdx.x) * kScanTile + u64(threadIdx.x) * kScanItems;
  u32 v[kScanItems];
  u64 s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
  {
    v[j] = base + j < n ? cnt[base + j] : 0u;
    s += v[j];
  }
  u64 total;
  u64 ex = block_scan_u64(s, ws, total) + tileSums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < kScanItems; ++j)
    if (base + j < n)
    {
      off[base + j] = ex;
      ex += v[j];
    }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    off[n] = tileSums[gridDim.x];
}

// warp per query: copies its entries from the append buffer (or the plain result) to CSR order
__global__ void csr_move_kernel(const u64* __restrict__ start, const u32* __restrict__ count, const u64* __restrict__ off, u64 nq,
                                const u32* __restrict__ ids, const double* __restrict__ dist, const u32* __restrict__ fbIds,
                                const double* __restrict__ fbDist, u32* __restrict__ outIds, double* __restrict__ outDist)
{
  const u32 lane = threadIdx.x & 31;
  for (u64 q = (blockIdx.x * u64(blockDim.x) + threadIdx.x) >> 5; q < nq; q += (u64(gridDim.x) * blockDim.x) >> 5)
  {
    const u32 c = count[q];
    if (!c)
      continue;
    const u64 s = start[q];
    const bool fb = (s >> 32) & kFromFallback;
    const u64 src = s & ~(u64(kFromFallback) << 32);
    const u32* si = fb ? fbIds : ids;
    const double* sd = fb ? fbDist : dist;
    const u64 d = off[q];
    for (u32 i = lane; i < c; i += 32)
    {
      outIds[d + i] = si[src + i];
      outDist[d + i] = sd[src + i];
    }
  }
}

// ---------------------------------------------------------------- host
static void host_bounds(double v, float& lo, float& hi)
{
  float f = float(v);
  lo = f;
  hi = f;
  if (double(f) > v)
    lo = std::nextafter(f, -kInf);
  if (double(f) < v)
    hi = std::nextafter(f, kInf);
}

template<typename T>
static int ensure_image32_impl(TreeState& t, cudaStream_t st)
{
  if (t.image32)
    return OTG_OK;
  cudaError_t e;
  if ((e = t.geom32.ensure(sizeof(float4) * std::max<u64>(t.n, 1))) || (e = t.nodeBox32.ensure(sizeof(float4) * 2 * std::max<u64>(t.nodeCount, 1))))
    return cuda_status(e, "allocating the FP32 tree image");
  if (t.kind == OTG_KIND_POINTS && t.n)
    point_image_kernel<T><<<blocks_for(t.n), 256, 0, st>>>(t.sortedGeom.as<T>(), t.n, t.geom32.as<float4>());
  node_image_kernel<T><<<blocks_for(t.nodeCount), 256, 0, st>>>(t.nodeBox.as<T>(), t.kind != OTG_KIND_POINTS ? t.nodeMax.as<T>() : nullptr, t.nodeCount,
                                                                 t.nodeBox32.as<float4>());
  if ((e = cudaGetLastError()))
    return cuda_status(e, "building the FP32 tree image");
  t.image32 = true;
  return OTG_OK;
}

template<typename T, int CAP, int WARPS>
static int launch_filtered_w(const KnnArgs<T>& a, cudaStream_t st)
{
  const size_t smem = sizeof(KnnWarpMem<CAP>) * WARPS;
  cudaError_t e = cudaFuncSetAttribute(knn_filtered_kernel<T, CAP, WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  int dev = 0, sms = 0, per = 0;
  if (!e)
    e = cudaGetDevice(&dev);
  if (!e)
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!e)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, knn_filtered_kernel<T, CAP, WARPS>, WARPS * 32, smem);
  if (e)
    return cuda_status(e, "configuring the kNN kernel");
  const u64 want = (u64(a.nq) + WARPS - 1) / WARPS;
  const u32 grid = u32(std::max<u64>(1, std::min<u64>(u64(sms) * std::max(per, 1), want)));
  knn_filtered_kernel<T, CAP, WARPS><<<grid, WARPS * 32, smem, st>>>(a);
  return cuda_status(cudaGetLastError(), "launching the kNN kernel");
}

// shape: warps per block (2, 4 or 8)
template<typename T, int CAP>
static int launch_filtered(const KnnArgs<T>& a, int shape, cudaStream_t st)
{
  if (shape == 2)
    return launch_filtered_w<T, CAP, 2>(a, st);
  if (shape == 8)
    return launch_filtered_w<T, CAP, 8>(a, st);
  return launch_filtered_w<T, CAP, 4>(a, st);
}

template<typename T>
static int knn_filtered_impl(TreeState& t, const T* pts, const u32* dk, u64 nq, u32 kAll, double maxDist, double tol, ResultState& r, cudaStream_t st)
{
  cudaError_t e;
  if (int rc = ensure_image32(t, st))
    return rc;
  const T tl = tol_of<T>(tol);
  const T F0 = maxDist < 0 ? Lim<T>::max() : upper_tol_host(T(maxDist), tl);
  // k statistics: the buffer size follows the largest k, the output guess the sum of k
  u32 kmax = kAll;
  u64 ksum = u64(kAll) * nq;
  TmpBuf stats;
  if (dk)
  {
    if ((e = stats.ensure(16, st)))
      return cuda_status(e, "allocating k statistics");
    cudaMemsetAsync(stats.p, 0, 16, st);
    k_stats_kernel<<<blocks_for(nq), 256, 0, st>>>(dk, nq, stats.as<u32>(), reinterpret_cast<unsigned long long*>(stats.as<unsigned char>() + 8));
    unsigned long long h[2] = { 0, 0 };
    e = cudaMemcpyAsync(h, stats.p, 16, cudaMemcpyDeviceToHost, st);
    if (!e)
      e = cudaStreamSynchronize(st);
    if (e)
      return cuda_status(e, "reading k statistics");
    kmax = u32(h[0]);
    ksum = h[1];
  }
  const bool big = kmax > 112;
  // spatial order of the queries
  TmpBuf qkeys, order;
  if ((e = qkeys.ensure(sizeof(u32) * nq, st)) || (e = order.ensure(sizeof(u32) * nq, st)))
    return cuda_status(e, "allocating the query order");
  // below 64k queries the batch takes the queries in input order: four radix passes over a few
  // tiles cost more than the locality gains, the tree's upper levels sitting in L2 anyway
  const bool sortQueries = nq >= (u64(1) << 16);
  if (sortQueries)
    query_key_kernel<T><<<blocks_for(nq), 256, 0, st>>>(pts, nq, t.space.as<Space<T>>(), qkeys.as<u32>(), order.as<u32>());
  else
    iota_order_kernel<<<blocks_for(nq), 256, 0, st>>>(order.as<u32>(), nq);
  TmpBuf ctr, fb, start, cnt, oIds, oDist;
  if ((e = ctr.ensure(sizeof(KnnCounters), st)) || (e = fb.ensure(sizeof(u32) * nq, st)) || (e = start.ensure(sizeof(u64) * nq, st)) ||
      (e = cnt.ensure(sizeof(u32) * nq, st)))
    return cuda_status(e, "allocating kNN buffers");
  cudaMemsetAsync(ctr.p, 0, sizeof(KnnCounters), st);
  if (sortQueries)
    if (int rc = sort_pairs_u32(qkeys.as<u32>(), order.as<u32>(), nq, 30, st, &ctr.as<KnnCounters>()->err))
      return rc;
  qkeys.release();
  KnnArgs<T> a{};
  a.link = t.nodeLink.as<uint4>();
  a.nodeBox32 = t.nodeBox32.as<float4>();
  a.geom32 = t.geom32.as<float4>();
  a.geom = t.sortedGeom.as<T>();
  a.ids = t.sortedIds.as<u32>();
  a.n = u32(t.n);
  a.nNodes = u32(t.nodeCount);
  a.pts = pts;
  a.kArr = dk;
  a.kAll = kAll;
  a.nq = u32(nq);
  a.order = order.as<u32>();
  a.F0 = F0;
  a.tol = tl;
  float lo, hi;
  host_bounds(double(F0), lo, hi);
  a.F0hi = hi;
  {
    float l2, h2;
    host_bounds(double(lo) * double(lo), l2, h2);
    a.F0lo2 = l2;
  }
  host_bounds(double(tl), lo, hi);
  a.tolHi = hi;
  host_bounds(double(T(T(1) + tl)), lo, hi);
  host_bounds(double(hi) * (1.0 + 0x1p-20), lo, hi); // margin for the rounding of one product
  a.onePlusTolHi = hi;
  // relative margins that cover the rounding of the exact distance formula
  a.widenLo = sizeof(T) == 8 ? 1.f - 0x1p-18f : 1.f - 0x1p-16f;
  a.widenHi = sizeof(T) == 8 ? 1.f + 0x1p-18f : 1.f + 0x1p-16f;
  a.kLimit = big ? 240u : 112u;
  a.ctr = ctr.as<KnnCounters>();
  a.fallback = fb.as<u32>();
  a.start = start.as<u64>();
  a.count = cnt.as<u32>();
  u64 cap = ksum + ksum / 8 + 4096;
  KnnCounters h{};
  for (int attempt = 0; attempt < 2; ++attempt)
  {
    if ((e = oIds.ensure(sizeof(u32) * cap, st)) || (e = oDist.ensure(sizeof(double) * cap, st)))
      return cuda_status(e, "allocating the kNN output");
    a.outIds = oIds.as<u32>();
    a.outDist = oDist.as<double>();
    a.outCap = cap;
    int rc = tune_run(tune_key("knn", sizeof(T) == 8, int(t.kind), t.n, nq), { { 2, "warp x2" }, { 4, "warp x4" }, { 8, "warp x8" } }, 4, st,
                      [&](int shape) {
                        cudaMemsetAsync(ctr.p, 0, offsetof(KnnCounters, err), st); // keeps the sort's error bits
                        return big ? launch_filtered<T, 512>(a, shape, st) : launch_filtered<T, 256>(a, shape, st);
                      });
    if (rc)
      return rc;
    e = cudaMemcpyAsync(&h, ctr.p, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (!e)
      e = cudaStreamSynchronize(st);
    if (e)
      return cuda_status(e, "running the kNN kernel");
    if (h.out <= cap)
      break;
    cap = h.out + h.out / 16 + 4096;
  }
  if (h.err & kErrTimeout)
  {
    set_error("a bounded device wait ran out");
    return OTG_ERR_TIMEOUT;
  }
  if (h.out > cap)
  {
    set_error("kNN output sizing did not converge");
    return OTG_ERR_OUT_OF_MEMORY;
  }
  // queries the filter handed over to the plain kernels
  ResultState fbr;
  if (h.fallbacks)
  {
    TmpBuf fpts, fk;
    if ((e = fpts.ensure(sizeof(T) * 3 * h.fallbacks, st)) || (e = fk.ensure(sizeof(u32) * h.fallbacks, st)))
      return cuda_status(e, "allocating fallback queries");
    fallback_points_kernel<<<blocks_for(h.fallbacks), 256, 0, st>>>(fb.as<u32>(), h.fallbacks, pts, u32(sizeof(T) * 3), dk, kAll,
                                                                   fpts.as<unsigned char>(), fk.as<u32>());
    if (int rc = query_knn(t, fpts.p, h.fallbacks, fk.as<u32>(), 0, maxDist, tol, OTG_ALGO_PLAIN_FP64, fbr, OTG_MEM_DEVICE, st))
      return rc;
    fallback_slots_kernel<<<blocks_for(h.fallbacks), 256, 0, st>>>(fb.as<u32>(), h.fallbacks, fbr.offsets.as<u64>(), start.as<u64>(), cnt.as<u32>());
  }
  // CSR: offsets by scan of the counts, then entries moved into query order
  const u64 tiles = (nq + kScanTile - 1) / kScanTile;
  TmpBuf tileSums;
  if ((e = tileSums.ensure(sizeof(u64) * (tiles + 1), st)) || (e = result_alloc(r, sizeof(u64) * (nq + 1), 0, 0, st)))
    return cuda_status(e, "allocating result offsets");
  scan_reduce_kernel<<<u32(tiles), kScanThreads, 0, st>>>(cnt.as<u32>(), nq, tileSums.as<u64>());
  scan_tiles_kernel<<<1, kScanThreads, 0, st>>>(tileSums.as<u64>(), tiles);
  scan_apply_kernel<<<u32(tiles), kScanThreads, 0, st>>>(cnt.as<u32>(), nq, tileSums.as<u64>(), r.offsets.as<u64>());
  const u64 total = h.out + fbr.nids;
  if ((e = result_alloc(r, 0, sizeof(u32) * std::max<u64>(total, 1), sizeof(double) * std::max<u64>(total, 1), st)))
    return cuda_status(e, "allocating the result");
  csr_move_kernel<<<blocks_for(nq * 32), 256, 0, st>>>(start.as<u64>(), cnt.as<u32>(), r.offsets.as<u64>(), nq, oIds.as<u32>(), oDist.as<double>(),
                                                        fbr.ids.as<u32>(), fbr.dist.as<double>(), r.ids.as<u32>(), r.dist.as<double>());
  e = cudaStreamSynchronize(st);
  if (e || (e = cudaGetLastError()))
    return cuda_status(e, "assembling the kNN result");
  r.nq = nq;
  r.nids = total;
  r.hasDist = true;
  r.filterTests = h.tests;
  r.rechecks = h.rechecks;
  return OTG_OK;
}

int ensure_image32(TreeState& t, cudaStream_t st)
{
  return t.scalar == OTG_SCALAR_F64 ? ensure_image32_impl<double>(t, st) : ensure_image32_impl<float>(t, st);
}

int knn_filtered(TreeState& t, const void* dpts, const u32* dk, u64 nq, u32 kAll, double maxDist, double tol, ResultState& r, cudaStream_t st)
{
  return t.scalar == OTG_SCALAR_F64 ? knn_filtered_impl<double>(t, (const double*)dpts, dk, nq, kAll, maxDist, tol, r, st)
                                    : knn_filtered_impl<float>(t, (const float*)dpts, dk, nq, kAll, maxDist, tol, r, st);
}

} // namespace otg
