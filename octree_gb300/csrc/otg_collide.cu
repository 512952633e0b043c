// otg_collide.cu — candidate search of CollisionDetection (core/ot_query.h:1308-1497 two trees,
// :1690-1914 one tree) with an FP32 filter.
//
// One warp per entity of the first tree walks the other tree (entities of shallow nodes first, as
// their walks are the longest; the rest are taken from a shared counter): a node is entered when
// its MBR may meet the box, its own entities are tested by the lanes in parallel (coalesced loads
// of their images), and its children are tested in parallel. The test runs on an FP32 image of both boxes rounded
// outward (minimum and maximum rounded down, and rounded up with the tolerance added), which
// decides GetBoxRelation (general.h:262-289) for all but rounding-level cases:
//   certainly overlapped  a.min + tol < b.max and b.min + tol < a.max hold in every dimension
//   certainly not         b.max + tol < a.min or a.max + tol < b.min holds in some dimension
// (the first is the "overlapped" branch of every dimension; the second makes that dimension
// "separated" or "adjacent", either of which excludes "overlapped"). The undecided rest is
// re-tested with the exact predicate in the tree's scalar type, so the candidate set equals
// {pairs with GetBoxRelation == Overlapped} exactly. In a single tree only pairs whose second
// position follows the first are searched, so each pair is tested once.
#include "otg_query.cuh"

namespace otg
{

constexpr int kPairBuf = 256;

struct CollideCounters
{
  unsigned long long tests;
  unsigned long long rechecks;
  u32 work;
  u32 pad;
};

// per entity 12 floats in 3 float4: minD xyz, maxD xyz (rounded down), minU xyz, maxU xyz (rounded up, + tol)
template<typename T>
__global__ void box_image_kernel(const T* __restrict__ geom, u64 n, float tolHi, float4* __restrict__ out)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    float v[12];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      const double mn = double(geom[i * 6 + c]), mx = double(geom[i * 6 + 3 + c]);
      v[c] = __double2float_rd(mn);
      v[3 + c] = __double2float_rd(mx);
      v[6 + c] = __fadd_ru(__double2float_ru(mn), tolHi);
      v[9 + c] = __fadd_ru(__double2float_ru(mx), tolHi);
    }
    out[3 * i] = make_float4(v[0], v[1], v[2], v[3]);
    out[3 * i + 1] = make_float4(v[4], v[5], v[6], v[7]);
    out[3 * i + 2] = make_float4(v[8], v[9], v[10], v[11]);
  }
}

// node MBRs for one call: {min rounded down, 0}, {max rounded up + tol rounded up, 0}
__global__ void node_tol_image_kernel(const float4* __restrict__ nodes32, u64 m, float tolHi, float4* __restrict__ out)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < m; i += u64(gridDim.x) * blockDim.x)
  {
    const float4 mx = nodes32[2 * i + 1];
    out[2 * i] = nodes32[2 * i];
    out[2 * i + 1] = make_float4(__fadd_ru(mx.x, tolHi), __fadd_ru(mx.y, tolHi), __fadd_ru(mx.z, tolHi), 0.f);
  }
}

struct BoxImg
{
  float mnD[3], mxD[3], mnU[3], mxU[3];
};

__device__ __forceinline__ BoxImg load_img(const float4* __restrict__ img, u32 i)
{
  const float4 a = img[3 * size_t(i)], b = img[3 * size_t(i) + 1], c = img[3 * size_t(i) + 2];
  BoxImg r;
  r.mnD[0] = a.x;
  r.mnD[1] = a.y;
  r.mnD[2] = a.z;
  r.mxD[0] = a.w;
  r.mxD[1] = b.x;
  r.mxD[2] = b.y;
  r.mnU[0] = b.z;
  r.mnU[1] = b.w;
  r.mnU[2] = c.x;
  r.mxU[0] = c.y;
  r.mxU[1] = c.z;
  r.mxU[2] = c.w;
  return r;
}

// 1: certainly overlapped, -1: certainly not, 0: undecided in FP32
__device__ __forceinline__ int img_relation(const BoxImg& a, const BoxImg& b)
{
  bool ov = true, sep = false;
#pragma unroll
  for (int c = 0; c < 3; ++c)
  {
    ov &= (a.mnU[c] < b.mxD[c]) & (b.mnU[c] < a.mxD[c]);
    sep |= (b.mxU[c] < a.mnD[c]) | (a.mxU[c] < b.mnD[c]);
  }
  return ov ? 1 : (sep ? -1 : 0);
}

template<typename T>
struct CollideArgs
{
  const float4* imgA;
  const T* geomA;
  u32 nA;
  const u32* order; // processing order of the A entities
  const u32* ownerA; // node holding each A entity (kNoOwner: none reachable, skipped)
  const float4* imgB;
  const T* geomB;
  const uint4* linkB;
  const float4* nodeB; // node MBRs of tree B: min rounded down, max + tol rounded up (2 float4 per node)
  u32 nB, nNodesB;
  float tolHi;
  T tol;
  int selfMode;
  int swapOut; // two trees searched from the second tree's entities: emit (walked position, entity position)
  Appender out;
  CollideCounters* ctr;
  u32* err;
};

template<typename T, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) collide_box_kernel(CollideArgs<T> a)
{
  __shared__ u32 stackMem[WARPS][kStack];
  __shared__ u64 pairMem[WARPS][kPairBuf];
  const u32 lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  u32* stack = stackMem[w];
  u64* pbuf = pairMem[w];
  const u32 lt = (1u << lane) - 1;
  unsigned long long tests = 0, rechecks = 0;
  for (;;)
  {
    u32 item = 0;
    if (lane == 0)
      item = atomicAdd(&a.ctr->work, 1u);
    item = __shfl_sync(~0u, item, 0);
    if (item >= a.nA)
      break;
    const u32 i = a.order ? a.order[item] : item;
    if (a.ownerA && a.ownerA[i] == kNoOwner)
      continue; // an entity that no node reachable from the root holds takes part in no pair
    const BoxImg me = load_img(a.imgA, i);
    u32 nbuf = 0;
    if (lane == 0)
      stack[0] = 0;
    __syncwarp();
    int sp = 1;
    u32 visits = 0;
    bool bad = false;
    while (sp > 0)
    {
      const u32 node = stack[--sp];
      __syncwarp();
      const uint4 L = a.linkB[node];
      if (L.z > a.nB || L.y > L.z || ++visits > a.nNodesB)
      {
        bad = true;
        break;
      }
      const u32 jb = a.selfMode ? max(L.y, i + 1) : L.y;
      for (u32 base = jb; base < L.z; base += 32)
      {
        const u32 j = base + lane;
        bool hit = false;
        if (j < L.z)
        {
          const int rel = img_relation(me, load_img(a.imgB, j));
          hit = rel == 1;
          if (rel == 0)
          {
            T ea[6], eb[6];
            load_box(a.geomA + u64(i) * 6, ea);
            load_box(a.geomB + u64(j) * 6, eb);
            hit = GeoD<T>::box_relation(ea, eb, a.tol) == -1;
            ++rechecks;
          }
          ++tests;
        }
        const u32 bal = __ballot_sync(~0u, hit);
        if (bal)
        {
          if (nbuf + 32 > kPairBuf)
          {
            unsigned long long b0 = 0;
            if (lane == 0)
              b0 = a.out.reserve(nbuf);
            b0 = __shfl_sync(~0u, b0, 0);
            for (u32 t = lane; t < nbuf; t += 32)
              if (b0 + t < a.out.capacity)
                a.out.items[b0 + t] = pbuf[t];
            __syncwarp();
            nbuf = 0;
          }
          if (hit)
            pbuf[nbuf + __popc(bal & lt)] = a.swapOut ? ((u64(j) << 32) | i) : ((u64(i) << 32) | j);
          nbuf += __popc(bal);
          __syncwarp();
        }
      }
      const u32 fc = L.x & kFirstChildMask, cc = L.x >> kChildShift;
      if (cc)
      {
        if (u64(fc) + cc > a.nNodesB || sp + int(cc) > kStack)
        {
          bad = true;
          break;
        }
        bool keep = false;
        if (lane < cc)
        {
          const u32 ch = fc + lane;
          const float4 mn = a.nodeB[2 * size_t(ch)], mx = a.nodeB[2 * size_t(ch) + 1];
          const float nmn[3] = { mn.x, mn.y, mn.z }, nmx[3] = { mx.x, mx.y, mx.z };
          keep = true;
#pragma unroll
          for (int c = 0; c < 3; ++c)
            keep &= !((nmx[c] < me.mnD[c]) | (me.mxU[c] < nmn[c]));
          if (keep && a.selfMode)
            keep = a.linkB[ch].w > i + 1; // the subtree holds a position after this entity
        }
        const u32 bal = __ballot_sync(~0u, keep);
        if (keep)
          stack[sp + __popc(bal & lt)] = fc + lane;
        sp += __popc(bal);
        __syncwarp();
      }
    }
    if (bad && lane == 0)
      atomicOr(a.err, kErrStack);
    if (nbuf)
    {
      unsigned long long b0 = 0;
      if (lane == 0)
        b0 = a.out.reserve(nbuf);
      b0 = __shfl_sync(~0u, b0, 0);
      for (u32 t = lane; t < nbuf; t += 32)
        if (b0 + t < a.out.capacity)
          a.out.items[b0 + t] = pbuf[t];
    }
    __syncwarp();
  }
  for (int o = 16; o > 0; o >>= 1)
  {
    tests += __shfl_xor_sync(~0u, tests, o);
    rechecks += __shfl_xor_sync(~0u, rechecks, o);
  }
  if (lane == 0)
  {
    atomicAdd(&a.ctr->tests, tests);
    atomicAdd(&a.ctr->rechecks, rechecks);
  }
}

// processing order: entities of shallow nodes (large boxes, long walks) first
__global__ void owner_depth_key_kernel(const u32* __restrict__ owner, const unsigned char* __restrict__ depth, u64 n, u32* __restrict__ keys,
                                       u32* __restrict__ idx)
{
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    const u32 o = owner[i];
    keys[i] = o == kNoOwner ? 31u : depth[o]; // entities in no node last (the collision skips them)
    idx[i] = u32(i);
  }
}

static void host_ru(double v, float& hi)
{
  float f = float(v);
  if (double(f) < v)
    f = std::nextafter(f, __builtin_huge_valf());
  hi = f;
}

template<typename T, int WARPS>
static int launch_collide(const CollideArgs<T>& a, cudaStream_t st)
{
  int dev = 0, sms = 0, per = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (!e)
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!e)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, collide_box_kernel<T, WARPS>, WARPS * 32, 0);
  if (e)
    return cuda_status(e, "configuring the collision kernel");
  const u32 grid = u32(std::max<u64>(1, std::min<u64>(u64(sms) * std::max(per, 1), (u64(a.nA) + WARPS - 1) / WARPS)));
  collide_box_kernel<T, WARPS><<<grid, WARPS * 32, 0, st>>>(a);
  return cuda_status(cudaGetLastError(), "launching the collision kernel");
}

// Per-call state of the filtered search: the tolerance-specific FP32 images of both trees.
template<typename T>
static int collide_search_impl(TreeState& A, TreeState& B, bool self, bool swapOut, double tol, Appender out, u32* err, CollideSearch& s,
                               cudaStream_t st)
{
  cudaError_t e;
  if (!s.ready)
  {
    if (int rc = ensure_image32(B, st))
      return rc;
    const T tl = tol < 0 ? base_tol<T>() : T(tol);
    host_ru(double(tl), s.tolHi);
    if ((e = s.imgA.ensure(sizeof(float4) * 3 * std::max<u64>(A.n, 1))) || (!self && (e = s.imgB.ensure(sizeof(float4) * 3 * std::max<u64>(B.n, 1)))) ||
        (e = s.ctr.ensure(sizeof(CollideCounters))) || (e = s.nodesB.ensure(sizeof(float4) * 2 * std::max<u64>(B.nodeCount, 1))))
      return cuda_status(e, "allocating the collision images");
    node_tol_image_kernel<<<blocks_for(B.nodeCount), 256, 0, st>>>(B.nodeBox32.as<float4>(), B.nodeCount, s.tolHi, s.nodesB.as<float4>());
    box_image_kernel<T><<<blocks_for(A.n), 256, 0, st>>>(A.sortedGeom.as<T>(), A.n, s.tolHi, s.imgA.as<float4>());
    if (!self)
      box_image_kernel<T><<<blocks_for(B.n), 256, 0, st>>>(B.sortedGeom.as<T>(), B.n, s.tolHi, s.imgB.as<float4>());
    s.ready = true;
  }
  if (!s.orderReady)
  {
    TmpBuf keys;
    if ((e = keys.ensure(sizeof(u32) * std::max<u64>(A.n, 1), st)) || (e = s.order.ensure(sizeof(u32) * std::max<u64>(A.n, 1))))
      return cuda_status(e, "allocating the collision order");
    owner_depth_key_kernel<<<blocks_for(A.n), 256, 0, st>>>(A.ownerNode.as<u32>(), A.nodeDepth.as<unsigned char>(), A.n, keys.as<u32>(), s.order.as<u32>());
    if (int rc = sort_pairs_u32(keys.as<u32>(), s.order.as<u32>(), A.n, 5, st, err))
      return rc;
    s.orderReady = true;
  }
  CollideArgs<T> a{};
  a.order = s.order.as<u32>();
  a.ownerA = A.ownerNode.as<u32>();
  a.imgA = s.imgA.as<float4>();
  a.geomA = A.sortedGeom.as<T>();
  a.nA = u32(A.n);
  a.imgB = self ? s.imgA.as<float4>() : s.imgB.as<float4>();
  a.geomB = B.sortedGeom.as<T>();
  a.linkB = B.nodeLink.as<uint4>();
  a.nodeB = s.nodesB.as<float4>();
  a.nB = u32(B.n);
  a.nNodesB = u32(B.nodeCount);
  a.tolHi = s.tolHi;
  a.tol = tol < 0 ? base_tol<T>() : T(tol);
  a.selfMode = self ? 1 : 0;
  a.swapOut = swapOut ? 1 : 0;
  a.out = out;
  a.ctr = s.ctr.as<CollideCounters>();
  a.err = err;
  return tune_run(tune_key(self ? "collide self" : "collide pair", sizeof(T) == 8, 1, B.n, A.n), { { 2, "warp x2" }, { 4, "warp x4" }, { 8, "warp x8" } }, 4,
                  st, [&](int shape) {
                    cudaMemsetAsync(s.ctr.p, 0, sizeof(CollideCounters), st);
                    cudaMemsetAsync(out.count, 0, sizeof(unsigned long long), st);
                    if (shape == 2)
                      return launch_collide<T, 2>(a, st);
                    if (shape == 8)
                      return launch_collide<T, 8>(a, st);
                    return launch_collide<T, 4>(a, st);
                  });
}

int collide_search_filtered(TreeState& A, TreeState& B, bool self, double tol, Appender out, u32* err, CollideSearch& s, cudaStream_t st)
{
  const bool swap = !self && B.n < A.n;
  TreeState& Q = swap ? B : A;
  TreeState& W = swap ? A : B;
  return A.scalar == OTG_SCALAR_F64 ? collide_search_impl<double>(Q, W, self, swap, tol, out, err, s, st)
                                    : collide_search_impl<float>(Q, W, self, swap, tol, out, err, s, st);
}

int collide_search_stats(const CollideSearch& s, u64& tests, u64& rechecks, cudaStream_t st)
{
  CollideCounters h{};
  cudaError_t e = cudaMemcpyAsync(&h, s.ctr.p, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (!e)
    e = cudaStreamSynchronize(st);
  if (e)
    return cuda_status(e, "reading collision statistics");
  tests = h.tests;
  rechecks = h.rechecks;
  return OTG_OK;
}

} // namespace otg
