// otg_sort_chunked.cuh — LSD radix sort of (key, u32 value) pairs in persistent, chunked passes.
//
// Replaces the reference's std::sort(par) over (Location, EntityID) in Create
// (core/ot_dynamic_hash_core.h:791-796) for single trees; the order is the same key order (stable:
// equal keys keep ascending entity id; the reference's unstable sort leaves them unspecified).
//
// Why chunked: a decoupled look-back pass publishes one prefix per tile, and each tile waits for
// the inclusive prefixes of the tiles before it. With hundreds of tiles in flight that chain of
// L2 round trips, not the bytes, sets the pass time. Here each CTA of a co-resident grid owns a
// contiguous chunk of tiles instead:
//   1. it counts the digits of its whole chunk (one read of the keys) and writes that histogram;
//   2. after a grid barrier, CTA c turns the digit columns c, c + G, ... into exclusive prefixes
//      over the chunks and writes the digit totals; after a second barrier every CTA has its
//      starting position per digit (digit start + the counts of earlier chunks);
//   3. it streams its tiles in order: the next tile's keys and values arrive in shared memory by
//      bulk copies (cp.async.bulk, completion on an mbarrier) while the current tile is ranked
//      (warp ballots, stable), staged in digit order and written out in runs, and its per-digit
//      positions advance by the tile's counts. No tile waits on another.
// Digits are 8-11 bits wide, so 31-bit point keys take 3 passes and 41-bit box keys 4.
// Every wait is bounded (grid barrier spins, mbarrier waits): on timeout the CTA sets an error bit,
// waits (bounded again) for its own copies in flight and returns, so the GPU is never held.
// The grid must be co-resident: it is launched as a cooperative kernel sized by the occupancy.
#pragma once

#include "otg_sort.cuh"

namespace otg
{
constexpr int kChunkThreads = 512;
constexpr int kChunkItems = 8;
constexpr int kChunkTile = kChunkThreads * kChunkItems; // 4096
constexpr int kChunkWarps = kChunkThreads / 32;
constexpr int kChunkMaxGrid = 512;   // the column scan gives one chunk per thread
constexpr int kChunkMaxBits = 11;    // widest digit
constexpr u32 kGridSpinLimit = 1u << 22;  // grid barrier spins (each with a short sleep)

// Grid barrier of a co-resident grid: arrival count `target` (monotonic counter per pass).
// Returns false (and sets the error bit) when the other CTAs do not arrive in time.
__device__ __forceinline__ bool grid_barrier(u32* counter, u32 target, u32* err, int* s_ok)
{
  __syncthreads();
  if (threadIdx.x == 0)
  {
    __threadfence();
    atomicAdd(counter, 1u);
    volatile u32* vc = counter;
    u32 spins = 0;
    int ok = 1;
    while (*vc < target)
    {
      if (++spins > kGridSpinLimit)
      {
        atomicOr(err, kErrTimeout);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

// exclusive scan over the block of one value per thread (kChunkWarps warps); returns the block total
__device__ __forceinline__ u32 chunk_block_scan(u32 v, u32* s_warp, u32& total)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    const u32 y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o)
      x += y;
  }
  if (lane == 31)
    s_warp[warp] = x;
  __syncthreads();
  if (warp == 0)
  {
    u32 w = lane < kChunkWarps ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      const u32 y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o)
        w += y;
    }
    if (lane < kChunkWarps)
      s_warp[lane] = w;
  }
  __syncthreads();
  const u32 r = (warp ? s_warp[warp - 1] : 0u) + x - v;
  total = s_warp[kChunkWarps - 1];
  __syncthreads();
  return r;
}

// Shared-memory layout of a pass (dynamic): two tile stages (keys then values), the warps' packed
// digit counters (two 16-bit counts per word), the per-digit positions of this CTA, two mbarriers.
template<typename K, int RB>
struct ChunkLayout
{
  static constexpr int R = 1 << RB;
  static constexpr int WORDS = R / 2;
  static constexpr size_t stage = size_t(kChunkTile) * (sizeof(K) + sizeof(u32));
  static constexpr size_t cnt = size_t(kChunkWarps) * WORDS * sizeof(u32);
  static constexpr size_t base = size_t(R) * sizeof(u32);
  static constexpr size_t bytes = 2 * stage + cnt + base + 2 * sizeof(u64);
};

// One pass: digit (key >> shift) & (2^RB - 1). vin == nullptr: values are the input positions.
// colHist: [G][2^RB] chunk histograms, then their column prefixes; digitTotal: [2^RB]; bar: this
// pass's barrier counter (zero at launch).
// CTAs per SM the kernel is compiled for: two for 32-bit keys and digits up to 10 bits (64
// registers, 105 KB of shared memory each), else one
template<typename K, int RB>
constexpr int chunk_min_blocks() { return (sizeof(K) == 4 && RB <= 10) ? 2 : 1; }

template<typename K, int RB>
__global__ void __launch_bounds__(kChunkThreads, chunk_min_blocks<K, RB>())
  chunk_sort_pass_kernel(const K* __restrict__ kin, const u32* __restrict__ vin, K* __restrict__ kout, u32* __restrict__ vout, u32 n, u32 shift,
                         u32* __restrict__ colHist, u32* __restrict__ digitTotal, u32* __restrict__ bar, u32* __restrict__ err)
{
  using L = ChunkLayout<K, RB>;
  constexpr int R = L::R;
  constexpr u32 MASK = u32(R - 1);
  constexpr int WORDS = L::WORDS;
  constexpr int WPT = (WORDS + kChunkThreads - 1) / kChunkThreads; // counter words owned per thread
  extern __shared__ __align__(16) unsigned char s_chunk[];
  u32* s_cnt = reinterpret_cast<u32*>(s_chunk + 2 * L::stage); // [kChunkWarps][WORDS]
  u32* s_base = reinterpret_cast<u32*>(s_chunk + 2 * L::stage + L::cnt);
  u64* s_bar = reinterpret_cast<u64*>(s_chunk + 2 * L::stage + L::cnt + L::base);
  __shared__ u32 s_warp[kChunkWarps];
  __shared__ int s_ok;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const u32 G = gridDim.x, c = blockIdx.x;
  const u32 tiles = (n + kChunkTile - 1) / kChunkTile;
  const u32 t0 = u32(u64(tiles) * c / G), t1 = u32(u64(tiles) * (c + 1) / G);
  const u32 e0 = t0 * u32(kChunkTile), e1 = min(n, t1 * u32(kChunkTile));

  // ---- 1. digit histogram of the chunk (the counter area doubles as the histogram)
  for (int d = tid; d < R; d += kChunkThreads)
    s_cnt[d] = 0;
  if (tid == 0)
  {
    mbar_init(&s_bar[0], 1);
    mbar_init(&s_bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if constexpr (sizeof(K) == 4)
  {
    const u32 v0 = e0 >> 2, v1 = e1 >> 2; // e0 is a multiple of 4: whole 16-byte words, then the tail
    const uint4* kv = reinterpret_cast<const uint4*>(kin);
    for (u32 i = v0 + tid; i < v1; i += kChunkThreads)
    {
      const uint4 w = kv[i];
      atomicAdd(&s_cnt[(w.x >> shift) & MASK], 1u);
      atomicAdd(&s_cnt[(w.y >> shift) & MASK], 1u);
      atomicAdd(&s_cnt[(w.z >> shift) & MASK], 1u);
      atomicAdd(&s_cnt[(w.w >> shift) & MASK], 1u);
    }
    for (u32 i = (v1 << 2) + tid; i < e1; i += kChunkThreads)
      atomicAdd(&s_cnt[u32(kin[i] >> shift) & MASK], 1u);
  }
  else
  {
    const u32 v0 = e0 >> 1, v1 = e1 >> 1;
    const ulonglong2* kv = reinterpret_cast<const ulonglong2*>(kin);
    for (u32 i = v0 + tid; i < v1; i += kChunkThreads)
    {
      const ulonglong2 w = kv[i];
      atomicAdd(&s_cnt[u32(w.x >> shift) & MASK], 1u);
      atomicAdd(&s_cnt[u32(w.y >> shift) & MASK], 1u);
    }
    for (u32 i = (v1 << 1) + tid; i < e1; i += kChunkThreads)
      atomicAdd(&s_cnt[u32(kin[i] >> shift) & MASK], 1u);
  }
  __syncthreads();
  for (int d = tid; d < R; d += kChunkThreads)
    colHist[u64(c) * R + d] = s_cnt[d];
  if (!grid_barrier(bar, G, err, &s_ok))
    return;

  // ---- 2. column prefixes over the chunks (CTA c takes digits c, c + G, ...), digit totals
  for (u32 d = c; d < u32(R); d += G)
  {
    const u32 x = tid < int(G) ? __ldcg(&colHist[u64(tid) * R + d]) : 0u;
    u32 tot;
    const u32 ex = chunk_block_scan(x, s_warp, tot);
    if (tid < int(G))
      colHist[u64(tid) * R + d] = ex;
    if (tid == 0)
      digitTotal[d] = tot;
  }
  if (!grid_barrier(bar, 2 * G, err, &s_ok))
    return;
  {
    // this CTA's position per digit: digit start (scan of the totals) + earlier chunks' counts
    constexpr int DPT = (R + kChunkThreads - 1) / kChunkThreads;
    u32 t[DPT], sum = 0;
#pragma unroll
    for (int j = 0; j < DPT; ++j)
    {
      const int d = tid * DPT + j;
      t[j] = d < R ? __ldcg(&digitTotal[d]) : 0u;
      sum += t[j];
    }
    u32 all;
    u32 start = chunk_block_scan(sum, s_warp, all);
#pragma unroll
    for (int j = 0; j < DPT; ++j)
    {
      const int d = tid * DPT + j;
      if (d < R)
        s_base[d] = start + __ldcg(&colHist[u64(c) * R + d]);
      start += t[j];
    }
  }
  __syncthreads();

  // ---- 3. the chunk's tiles in order, the next one arriving by bulk copies meanwhile
  auto tile_full = [&](u32 t) { return u64(t + 1) * kChunkTile <= u64(n); };
  auto stage_of = [&](u32 s) { return s_chunk + (s ? L::stage : size_t(0)); };
  auto issue = [&](u32 t, u32 s) {
    // thread 0: whole tiles only (16-byte multiples); the caller fenced the stage's earlier use
    const u32 b = t * u32(kChunkTile);
    const u32 bytes = vin ? u32(L::stage) : u32(sizeof(K) * kChunkTile);
    u64* mb = s_bar + s;
    mbar_arrive_expect_tx(mb, bytes);
    bulk_load(stage_of(s), kin + b, u32(sizeof(K) * kChunkTile), mb);
    if (vin)
      bulk_load(stage_of(s) + sizeof(K) * kChunkTile, vin + b, u32(sizeof(u32) * kChunkTile), mb);
  };
  // per stage s (bit s): the parity of its next mbarrier phase, and whether a copy is in flight
  u32 phaseBits = 0, inflightBits = 0;
  if (tid == 0 && t0 < t1 && tile_full(t0))
  {
    fence_proxy_async();
    issue(t0, 0);
  }
  if (t0 < t1 && tile_full(t0))
    inflightBits = 1;

  const u32 ltmask = lanemask_lt();
  bool failed = false;
  for (u32 t = t0, k = 0; t < t1; ++t, ++k)
  {
    const u32 s = k & 1u;
    K* sk = reinterpret_cast<K*>(stage_of(s));
    u32* sv = reinterpret_cast<u32*>(stage_of(s) + sizeof(K) * kChunkTile);
    const u32 base = t * u32(kChunkTile);
    const u32 count = min(u32(kChunkTile), n - base);
    if ((inflightBits >> s) & 1u)
    {
      // every thread waits on the mbarrier (which makes the copied bytes visible to it); the
      // outcome is made uniform so that no thread leaves the loop alone
      const bool ok = mbar_wait_bounded(s_bar + s, (phaseBits >> s) & 1u);
      if (__syncthreads_or(!ok))
      {
        failed = true;
        break;
      }
      phaseBits ^= 1u << s;
      inflightBits &= ~(1u << s);
    }
    else
    {
      // the partial last tile: plain loads
      for (u32 j = tid; j < count; j += kChunkThreads)
      {
        sk[j] = kin[base + j];
        if (vin)
          sv[j] = vin[base + j];
      }
    }
    // the next tile of the chunk into the other stage (its last use ended with the barrier below)
    if (t + 1 < t1 && tile_full(t + 1))
    {
      if (tid == 0)
      {
        fence_proxy_async();
        issue(t + 1, s ^ 1u);
      }
      inflightBits |= 1u << (s ^ 1u);
    }
    for (int i = tid; i < kChunkWarps * WORDS; i += kChunkThreads)
      s_cnt[i] = 0;
    __syncthreads();

    K keys[kChunkItems];
    u32 vals[kChunkItems], dig[kChunkItems];
    const u32 wb = u32(warp) * (32 * kChunkItems);
#pragma unroll
    for (int i = 0; i < kChunkItems; ++i)
    {
      const u32 j = wb + i * 32 + lane;
      const bool valid = j < count;
      keys[i] = valid ? sk[j] : K(0);
      vals[i] = vin ? (valid ? sv[j] : 0u) : base + j;
      dig[i] = valid ? u32((keys[i] >> shift) & MASK) : u32(R);
    }
    u32* wcnt = s_cnt + warp * WORDS;
#pragma unroll
    for (int i = 0; i < kChunkItems; ++i)
      if (dig[i] < u32(R))
        atomicAdd(&wcnt[dig[i] >> 1], 1u << (16 * (dig[i] & 1)));
    __syncthreads();

    // per owned word (two digits): warp offsets within the digit, tile totals
    u32 tot[WPT]; // packed tile counts of the owned words
    u32 mySum = 0;
#pragma unroll
    for (int j = 0; j < WPT; ++j)
    {
      const int w = tid * WPT + j;
      u32 acc = 0;
      if (w < WORDS)
      {
#pragma unroll
        for (int q = 0; q < kChunkWarps; ++q)
        {
          const u32 v = s_cnt[q * WORDS + w];
          s_cnt[q * WORDS + w] = acc;
          acc += v; // both halves stay below 2^16: a tile holds 4096 keys
        }
      }
      tot[j] = acc;
      mySum += (acc & 0xffffu) + (acc >> 16);
    }
    u32 tileTotal;
    u32 start = chunk_block_scan(mySum, s_warp, tileTotal);
    u32 startPacked[WPT];
#pragma unroll
    for (int j = 0; j < WPT; ++j)
    {
      const u32 lo = start, hi = start + (tot[j] & 0xffffu);
      startPacked[j] = lo | (hi << 16);
      start = hi + (tot[j] >> 16);
      const int w = tid * WPT + j;
      if (w < WORDS)
#pragma unroll
        for (int q = 0; q < kChunkWarps; ++q)
          s_cnt[q * WORDS + w] += startPacked[j];
    }
    __syncthreads();

    // stable rank: lanes sharing a digit found with one ballot per digit bit
    u32 pos[kChunkItems];
#pragma unroll
    for (int i = 0; i < kChunkItems; ++i)
    {
      const u32 d = dig[i];
      u32 peers = __ballot_sync(0xffffffffu, d < u32(R));
#pragma unroll
      for (int b = 0; b < RB; ++b)
      {
        const u32 bal = __ballot_sync(0xffffffffu, (d >> b) & 1u);
        peers &= ((d >> b) & 1u) ? bal : ~bal;
      }
      if (d >= u32(R))
        peers = 1u << lane;
      const int leader = __ffs(peers) - 1;
      u32 old = 0;
      if (d < u32(R) && lane == leader)
        old = atomicAdd(&wcnt[d >> 1], u32(__popc(peers)) << (16 * (d & 1)));
      old = __shfl_sync(0xffffffffu, old, leader);
      pos[i] = ((old >> (16 * (d & 1))) & 0xffffu) + __popc(peers & ltmask);
    }
    __syncthreads(); // every item of the stage is in registers: the stage takes the ranked tile
#pragma unroll
    for (int i = 0; i < kChunkItems; ++i)
      if (dig[i] < u32(R))
      {
        const u32 p = pos[i] & (kChunkTile - 1);
        sk[p] = keys[i];
        sv[p] = vals[i];
      }
    // tile-local start of each digit into the first warp's counter row (read by the write-out)
#pragma unroll
    for (int j = 0; j < WPT; ++j)
    {
      const int w = tid * WPT + j;
      if (w < WORDS)
        s_cnt[w] = startPacked[j];
    }
    __syncthreads();
    for (u32 j = tid; j < count; j += kChunkThreads)
    {
      const K key = sk[j];
      const u32 d = u32(key >> shift) & MASK;
      const u32 ts = (s_cnt[d >> 1] >> (16 * (d & 1))) & 0xffffu;
      const u32 p = s_base[d] + (j - ts);
      if (p < n)
      {
        kout[p] = key;
        vout[p] = sv[j];
      }
      else
        atomicOr(err, kErrTimeout);
    }
    __syncthreads();
    // positions advance by the tile's counts (each thread its own digits)
#pragma unroll
    for (int j = 0; j < WPT; ++j)
    {
      const int w = tid * WPT + j;
      if (w < WORDS)
      {
        s_base[2 * w] += tot[j] & 0xffffu;
        s_base[2 * w + 1] += tot[j] >> 16;
      }
    }
    // the next iteration's first barrier orders these updates before their readers
  }
  if (failed)
  {
    if (tid == 0)
      atomicOr(err, kErrTimeout);
    // let copies still in flight into this CTA's shared memory land before it exits
    for (u32 s = 0; s < 2; ++s)
      if ((inflightBits >> s) & 1u)
        mbar_wait_bounded(s_bar + s, (phaseBits >> s) & 1u);
  }
}

// Scratch of the chunked passes: chunk histograms [kChunkMaxGrid][2^kChunkMaxBits], digit totals,
// one barrier counter per pass (zeroed before the sort).
struct ChunkScratch
{
  u32* colHist = nullptr;
  u32* digitTotal = nullptr;
  u32* bars = nullptr;
  static constexpr int kMaxPasses = 8;
  static size_t bytes() { return sizeof(u32) * (size_t(kChunkMaxGrid) * (1u << kChunkMaxBits) + (1u << kChunkMaxBits) + kMaxPasses); }
  static size_t zero_offset() { return sizeof(u32) * (size_t(kChunkMaxGrid) * (1u << kChunkMaxBits) + (1u << kChunkMaxBits)); }
  static size_t zero_bytes() { return sizeof(u32) * kMaxPasses; }
  void carve(void* p)
  {
    u32* q = reinterpret_cast<u32*>(p);
    colHist = q;
    q += size_t(kChunkMaxGrid) * (1u << kChunkMaxBits);
    digitTotal = q;
    q += (1u << kChunkMaxBits);
    bars = q;
  }
};

// digit widths (low digit first) of a sort over `bits` key bits: as few passes of at most 11 bits
// as possible, widths as even as possible (31 bits: 11, 10, 10; 41: 11, 10, 10, 10)
inline int chunk_pass_widths(u32 bits, int* widths, int maxBits = kChunkMaxBits)
{
  maxBits = std::clamp(maxBits, 8, kChunkMaxBits);
  const int passes = std::max(1, int((bits + maxBits - 1) / maxBits));
  const int w = int(bits) / passes, extra = int(bits) % passes;
  for (int p = 0; p < passes; ++p)
    widths[p] = std::max(8, w + (p < extra ? 1 : 0));
  return passes;
}

template<typename K, int RB>
inline int chunk_pass_launch(const K* ki, const u32* vi, K* ko, u32* vo, u32 n, u32 shift, ChunkScratch& s, int pass, u32* err, cudaStream_t st)
{
  using L = ChunkLayout<K, RB>;
  auto kern = chunk_sort_pass_kernel<K, RB>;
  static int gridOf[64] = {}; // co-resident CTAs of this kernel per device (queried once)
  int dev = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)))
    return cuda_status(e, "querying the current device");
  int& grid = gridOf[dev & 63];
  if (!grid)
  {
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L::bytes))))
      return cuda_status(e, "configuring the sort pass");
    int sms = 0, perSm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, kChunkThreads, L::bytes)))
      return cuda_status(e, "sizing the sort pass");
    if (perSm < 1)
    {
      set_error("the sort pass does not fit on a multiprocessor");
      return OTG_ERR_NOT_SUPPORTED;
    }
    grid = std::min(kChunkMaxGrid, sms * perSm);
  }
  const u32 tiles = (n + kChunkTile - 1) / kChunkTile;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(std::max(1u, std::min(u32(grid), tiles)));
  cfg.blockDim = dim3(kChunkThreads);
  cfg.dynamicSmemBytes = L::bytes;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, kern, ki, vi, ko, vo, n, shift, s.colHist, s.digitTotal, s.bars + pass, err), "launching a sort pass");
}

// All passes over `bits` key bits. Pass p reads buffer (p even ? 0 : 1) and writes the other;
// *inB = the result is in (k1, v1). iotaValues: the first pass generates the values 0..n-1.
// s.bars must be zero (the caller clears ChunkScratch::zero_bytes at zero_offset).
template<typename K>
inline int chunk_sort(K* k0, u32* v0, K* k1, u32* v1, u64 n, u32 bits, bool iotaValues, ChunkScratch& s, u32* err, cudaStream_t st, bool* inB,
                      int maxBits = kChunkMaxBits)
{
  int widths[ChunkScratch::kMaxPasses];
  const int passes = chunk_pass_widths(bits, widths, maxBits);
  u32 shift = 0;
  for (int p = 0; p < passes; ++p)
  {
    const bool even = (p % 2) == 0;
    const K* ki = even ? k0 : k1;
    const u32* vi = (p == 0 && iotaValues) ? nullptr : (even ? v0 : v1);
    K* ko = even ? k1 : k0;
    u32* vo = even ? v1 : v0;
    int rc;
    switch (widths[p])
    {
    case 8: rc = chunk_pass_launch<K, 8>(ki, vi, ko, vo, u32(n), shift, s, p, err, st); break;
    case 9: rc = chunk_pass_launch<K, 9>(ki, vi, ko, vo, u32(n), shift, s, p, err, st); break;
    case 10: rc = chunk_pass_launch<K, 10>(ki, vi, ko, vo, u32(n), shift, s, p, err, st); break;
    default: rc = chunk_pass_launch<K, 11>(ki, vi, ko, vo, u32(n), shift, s, p, err, st); break;
    }
    if (rc)
      return rc;
    shift += u32(widths[p]);
  }
  *inB = (passes % 2) == 1;
  return OTG_OK;
}

} // namespace otg
