// otg_sort.cuh — single-pass-per-digit ("onesweep") LSD radix sort of (key, u32 value) pairs.
//
// Sorting replaces the reference's std::sort(par) over (Location, EntityID) in Create
// (core/ot_dynamic_hash_core.h:791-796); the result is the same key order (the reference's
// sort is unstable, this one is stable, so equal keys keep ascending entity id).
//
// Per pass, every CTA takes the next tile id from a counter (so tiles start in launch order),
// loads its tile's keys and values (or, with OTG_SORT_STAGE=1, receives whole tiles by bulk copies,
// cp.async.bulk into shared memory completing on an mbarrier), counts its 4096 keys per digit and
// publishes the counts, ranks the keys stably with warp
// ballots, looks back over earlier tiles' published counts (decoupled look-back) to get its global
// offsets, stages the tile in shared memory in digit order and writes it out in runs. Look-back spins are bounded:
// on timeout the CTA sets an error bit and finishes, so a broken invariant can never hang the GPU.
#pragma once

#include <cstdlib>

#include "otg_device.cuh"

namespace otg
{
constexpr int kSortThreads = 512;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems; // 4096
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr u32 kStatusAggregate = 1u << 30;
constexpr u32 kStatusInclusive = 2u << 30;
constexpr u32 kStatusValueMask = (1u << 30) - 1;
constexpr u32 kLookbackSpinLimit = 1u << 22;
constexpr int kLookbackBatch = 8;

// error bits reported by device code
constexpr u32 kErrTimeout = 1u;
constexpr u32 kErrCapacity = 2u;
constexpr u32 kErrStack = 4u;
constexpr u32 kErrArgument = 8u; // an input index out of range (reported, never followed)

// ---- bulk copies (cp.async.bulk) into shared memory, completing on an mbarrier
constexpr u32 kCopySpinLimit = 1u << 20; // mbarrier polls for one tile's bulk copies

__device__ __forceinline__ u32 smem_addr(const void* p) { return u32(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(u64* bar, u32 count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(u64* bar, u32 bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// true once the phase of the given parity has completed
__device__ __forceinline__ bool mbar_try_wait(u64* bar, u32 parity)
{
  u32 done;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
               : "=r"(done)
               : "r"(smem_addr(bar)), "r"(parity)
               : "memory");
  return done != 0;
}

// bulk copy global -> this CTA's shared memory (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_load(void* dst, const void* src, u32 bytes, u64* bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)), "l"(src), "r"(bytes),
               "r"(smem_addr(bar))
               : "memory");
}

// orders this thread's earlier generic-proxy shared-memory accesses before later bulk copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// bounded wait for the phase `parity` of bar, by every thread; false on timeout
__device__ __forceinline__ bool mbar_wait_bounded(u64* bar, u32 parity)
{
  for (u32 spins = 0; spins < kCopySpinLimit; ++spins)
    if (mbar_try_wait(bar, parity))
      return true;
  return false;
}

__device__ __forceinline__ u32 lanemask_lt()
{
  u32 m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// exclusive scan of one value per thread over the block (kSortWarps warps); returns the block total
__device__ __forceinline__ u32 block_exclusive_scan(u32 v, u32* s_warp, u32& total)
{
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    u32 y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o)
      x += y;
  }
  if (lane == 31)
    s_warp[warp] = x;
  __syncthreads();
  if (warp == 0)
  {
    u32 w = lane < kSortWarps ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
      u32 y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o)
        w += y;
    }
    if (lane < kSortWarps)
      s_warp[lane] = w; // inclusive warp totals
  }
  __syncthreads();
  u32 warpPrefix = warp ? s_warp[warp - 1] : 0;
  total = s_warp[kSortWarps - 1];
  u32 r = warpPrefix + x - v;
  __syncthreads();
  return r;
}

// All-pass digit histograms of `keys` (shift0 + 8p for p < passes) accumulated into hist[p][256].
// nDev (optional): the element count in device memory (at most n), for launches recorded before
// the count is known (graph replay)
template<typename K>
__global__ void __launch_bounds__(256) radix_histogram_kernel(const K* __restrict__ keys, u64 n, u32 shift0, u32 passes, u32* __restrict__ hist,
                                                             const unsigned long long* __restrict__ nDev = nullptr)
{
  if (nDev)
    n = min(n, u64(*nDev));
  __shared__ u32 sh[8][kRadix];
  for (int i = threadIdx.x; i < 8 * kRadix; i += blockDim.x)
    (&sh[0][0])[i] = 0;
  __syncthreads();
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    K k = keys[i];
    for (u32 p = 0; p < passes; ++p)
      atomicAdd(&sh[p][(k >> (shift0 + kRadixBits * p)) & (kRadix - 1)], 1u);
  }
  __syncthreads();
  for (u32 p = 0; p < passes; ++p)
    for (int d = threadIdx.x; d < kRadix; d += blockDim.x)
      if (sh[p][d])
        atomicAdd(&hist[p * kRadix + d], sh[p][d]);
}

// Rows of 256 digit counts (one per pass, or per pass and segment) turned into their exclusive
// prefix sums in place: the global base of every digit, scanned once per pass instead of in every
// tile.
static __global__ void __launch_bounds__(kRadix) digit_base_kernel(u32* __restrict__ hist)
{
  __shared__ u32 s_warp[kRadix / 32];
  u32* row = hist + u64(blockIdx.x) * kRadix;
  const int d = threadIdx.x, lane = d & 31, warp = d >> 5;
  const u32 v = row[d];
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
  u32 before = 0;
#pragma unroll
  for (int w = 0; w < kRadix / 32; ++w)
    before += w < warp ? s_warp[w] : 0u;
  row[d] = before + x - v;
}

// Decoupled look-back for digit d of tile `tile`: the sum of the counts of the earlier tiles
// (down to firstTile) from their published statuses, eight predecessors per round trip. A wait
// that runs out of its iteration limit sets kErrTimeout and returns what it has.
__device__ __forceinline__ u32 lookback_prefix(volatile u32* vstatus, u32 tile, u32 firstTile, u32 d, u32* err)
{
  u32 prefix = 0;
  long long j = (long long)tile - 1;
  u32 spins = 0;
  while (j >= (long long)firstTile)
  {
    u32 sv[kLookbackBatch];
#pragma unroll
    for (int k = 0; k < kLookbackBatch; ++k)
      sv[k] = (j - k >= (long long)firstTile) ? vstatus[u64(j - k) * kRadix + d] : u32(kStatusInclusive);
    int used = 0;
    bool done = false;
#pragma unroll
    for (int k = 0; k < kLookbackBatch; ++k)
    {
      if (done || used < k)
        continue;
      const u32 flag = sv[k] & ~kStatusValueMask;
      if (flag == 0)
        continue; // not published yet: re-read from here
      prefix += sv[k] & kStatusValueMask;
      used = k + 1;
      done = flag == kStatusInclusive;
    }
    if (done)
      break;
    j -= used;
    if (used < kLookbackBatch)
    {
      if (++spins > kLookbackSpinLimit)
      {
        atomicOr(err, kErrTimeout);
        break;
      }
      __nanosleep(32);
    }
  }
  return prefix;
}

// One onesweep pass. vin == nullptr means values are the input positions (iota).
// Order of work in a tile: per-warp digit counts (shared-memory atomics without return values),
// publication of the tile's counts as an aggregate right away, then the ranking, and only then
// the look-back: predecessors have had the ranking's duration to publish their inclusive prefixes.
// Ranking is stable: a warp finds the lanes sharing its digit with eight ballots (one per digit
// bit), the group leader advances the warp's position cursor for that digit with one shared
// atomic, and each lane adds its rank among lower lanes.
// Segmented form (segTiles != null): independent sorts of the segments [segOff[s], segOff[s+1])
// in one launch. Tile i covers tile segTiles[i].y of segment segTiles[i].x (the tiles of a segment
// are consecutive, in order), the look-back stops at the segment's first tile, and digitBase holds
// 256 digit bases per segment. Positions are below 2^30, so they are kept in 32 bits.
// DEVN: the element count is read from device memory (segOff[0] as unsigned long long, at most n);
// tiles that start past it end at once (no later tile looks back at them).
// digitBase: the pass's global digit bases (digit_base_kernel), per segment in the segmented form
// (16M points: 0.444 ms for the four passes, against 0.453 ms scanning the counts in every tile).
// STAGE (single sort only): whole tiles arrive by bulk copies instead of plain loads. Measured on
// 16M points (4 passes, 31-bit keys): 0.522 ms staged against 0.517 ms with plain loads, so plain
// loads are the default and OTG_SORT_STAGE=1 selects the staged form.
template<typename K, bool SEG = false, bool DEVN = false, bool STAGE = false>
__global__ void __launch_bounds__(kSortThreads, 3) onesweep_pass_kernel(const K* __restrict__ kin, const u32* __restrict__ vin, K* __restrict__ kout,
                                                                     u32* __restrict__ vout, u32 n, u32 shift, const u32* __restrict__ digitBase,
                                                                     u32* __restrict__ status, u32* __restrict__ tileCounter, u32* __restrict__ err,
                                                                     const uint2* __restrict__ segTiles = nullptr, const u64* __restrict__ segOff = nullptr)
{
  extern __shared__ __align__(16) unsigned char s_dyn[];
  K* s_keys = reinterpret_cast<K*>(s_dyn);
  u32* s_vals = reinterpret_cast<u32*>(s_dyn + sizeof(K) * kSortTile);
  __shared__ u32 s_cnt[kSortWarps][kRadix]; // warp digit counts, then tile-local position cursors
  __shared__ u32 s_globalBase[kRadix];
  __shared__ u32 s_scan[kSortWarps];
  __shared__ u32 s_tile;
  __shared__ __align__(8) u64 s_bar; // completion of the tile's bulk copies

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0)
  {
    s_tile = atomicAdd(tileCounter, 1u);
    if constexpr (STAGE && !SEG && !DEVN)
    {
      mbar_init(&s_bar, 1);
      fence_mbar_init();
    }
  }
  for (int i = tid; i < kSortWarps * kRadix; i += kSortThreads)
    (&s_cnt[0][0])[i] = 0;
  __syncthreads();
  const u32 tile = s_tile;
  // segment of this tile: [segBase, segEnd), its digit counts, its first tile
  u32 segBase = 0, segEnd = n, tileInSeg = tile;
  if constexpr (DEVN)
  {
    segEnd = u32(min(u64(n), u64(*reinterpret_cast<const unsigned long long*>(segOff))));
    if (u64(tile) * kSortTile >= segEnd)
      return;
  }
  if constexpr (SEG)
  {
    const uint2 st = segTiles[tile];
    segBase = u32(segOff[st.x]);
    segEnd = u32(segOff[st.x + 1]);
    tileInSeg = st.y;
    digitBase += u64(st.x) * kRadix;
  }
  const u32 base = segBase + tileInSeg * u32(kSortTile);
  const u32 firstTile = tile - tileInSeg;

  K keys[kSortItems];
  u32 vals[kSortItems];
  u32 dig[kSortItems];
  const u32 wbase = base + u32(warp) * (32 * kSortItems);
  // A whole tile of the single sort arrives by bulk copies (16-byte aligned: tiles start at
  // multiples of 4096 elements of buffers from cudaMalloc) into the staging area, which takes the
  // digit-ordered tile later; a partial last tile and the segmented / device-count forms read
  // global memory directly. One load loop serves both through generic pointers.
  const K* ksrc = kin + wbase;
  const u32* vsrc = vin ? vin + wbase : nullptr;
  if constexpr (STAGE && !SEG && !DEVN)
  {
    if (u64(base) + kSortTile <= u64(segEnd))
    {
      if (tid == 0)
      {
        const u32 bytes = u32(sizeof(K) * kSortTile) + (vin ? u32(sizeof(u32) * kSortTile) : 0u);
        mbar_arrive_expect_tx(&s_bar, bytes);
        bulk_load(s_keys, kin + base, u32(sizeof(K) * kSortTile), &s_bar);
        if (vin)
          bulk_load(s_vals, vin + base, u32(sizeof(u32) * kSortTile), &s_bar);
      }
      // every thread waits on the mbarrier, which makes the copied bytes visible to it; copies that
      // do not complete in time leave the tile unsorted (the error bit fails the sort)
      const bool ok = mbar_wait_bounded(&s_bar, 0);
      if (__syncthreads_or(!ok))
      {
        if (tid == 0)
          atomicOr(err, kErrTimeout);
        mbar_wait_bounded(&s_bar, 0); // the copies land before this CTA's shared memory goes away
        return;
      }
      ksrc = s_keys + (wbase - base);
      vsrc = vin ? s_vals + (wbase - base) : nullptr;
    }
  }
#pragma unroll
  for (int i = 0; i < kSortItems; ++i)
  {
    const u32 idx = wbase + i * 32 + lane;
    const bool valid = idx < segEnd;
    keys[i] = valid ? ksrc[i * 32 + lane] : K(0);
    vals[i] = vsrc ? (valid ? vsrc[i * 32 + lane] : 0u) : idx;
    dig[i] = valid ? u32((keys[i] >> shift) & (kRadix - 1)) : u32(kRadix);
  }
#pragma unroll
  for (int i = 0; i < kSortItems; ++i)
    if (dig[i] < kRadix)
      atomicAdd(&s_cnt[warp][dig[i]], 1u);
  __syncthreads();

  // per digit (thread tid < 256 owns digit tid): warp offsets, the tile total, early publication
  u32 total = 0;
  volatile u32* vstatus = status;
  if (tid < kRadix)
  {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w)
    {
      u32 c = s_cnt[w][tid];
      s_cnt[w][tid] = total;
      total += c;
    }
    vstatus[u64(tile) * kRadix + tid] = (tileInSeg == 0 ? kStatusInclusive : kStatusAggregate) | total;
  }
  u32 tileTotal;
  const u32 digitStart = block_exclusive_scan(total, s_scan, tileTotal);
  if (tid < kRadix)
  {
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w)
      s_cnt[w][tid] += digitStart;
  }
  __syncthreads();

  // Ranking, and each key straight into shared memory at its rank in the tile's digit order (the
  // loads from a staged tile ended at the barrier after the counts), so the look-back holds no keys
  // in registers. 16M points, the four passes: 0.453 ms, against 0.498 ms scattering from a rank
  // array after the ranking and 0.515 ms scattering after the look-back.
  const u32 ltmask = lanemask_lt();
#pragma unroll
  for (int i = 0; i < kSortItems; ++i)
  {
    const u32 d = dig[i];
    u32 peers = __ballot_sync(0xffffffffu, d < kRadix);
#pragma unroll
    for (int b = 0; b < kRadixBits; ++b)
    {
      const u32 bal = __ballot_sync(0xffffffffu, (d >> b) & 1u);
      peers &= ((d >> b) & 1u) ? bal : ~bal;
    }
    if (d >= kRadix)
      peers = 1u << lane;
    const int leader = __ffs(peers) - 1;
    u32 old = 0;
    if (d < kRadix && lane == leader)
      old = atomicAdd(&s_cnt[warp][d], u32(__popc(peers)));
    old = __shfl_sync(0xffffffffu, old, leader);
    if (d < kRadix)
    {
      const u32 p = (old + __popc(peers & ltmask)) & (kSortTile - 1); // ranks of a tile are below kSortTile by construction
      s_keys[p] = keys[i];
      s_vals[p] = vals[i];
    }
  }

  // The look-back after the ranking: predecessors have had the ranking's duration to publish
  // (looking back first, beside the other warps' ranking: 0.447 against 0.444 ms). Eight
  // predecessors per round trip measured best (16: 0.511 ms, 32: 0.562 ms, before the changes above).
  u32 prefix = 0;
  if (tid < kRadix && tileInSeg > 0)
  {
    prefix = lookback_prefix(vstatus, tile, firstTile, u32(tid), err);
    vstatus[u64(tile) * kRadix + tid] = kStatusInclusive | ((prefix + total) & kStatusValueMask);
  }
  if (tid < kRadix)
    s_globalBase[tid] = segBase + digitBase[tid] + prefix - digitStart;
  __syncthreads();

  const u32 tileCount = min(u32(kSortTile), segEnd - base);
  for (u32 j = tid; j < tileCount; j += kSortThreads)
  {
    const K k = s_keys[j];
    const u32 p = s_globalBase[u32((k >> shift) & (kRadix - 1))] + j;
    if (p - segBase < segEnd - segBase)
    {
      kout[p] = k;
      vout[p] = s_vals[j];
    }
    else
      atomicOr(err, kErrTimeout);
  }
}

// Scratch for a sort of up to n keys over `passes` digits.
struct SortScratch
{
  u32* hist = nullptr;        // passes * 256
  u32* status = nullptr;      // passes * tiles * 256
  u32* tileCounters = nullptr; // passes
  static size_t tiles(u64 n) { return size_t((n + kSortTile - 1) / kSortTile); }
  static size_t bytes(u64 n, u32 passes) { return sizeof(u32) * (size_t(passes) * kRadix + size_t(passes) * tiles(n) * kRadix + passes + 8); }
  void carve(void* p, u64 n, u32 passes)
  {
    u32* q = reinterpret_cast<u32*>(p);
    hist = q;
    q += size_t(passes) * kRadix;
    status = q;
    q += size_t(passes) * tiles(n) * kRadix;
    tileCounters = q;
  }
};

template<typename K>
inline size_t onesweep_smem_bytes()
{
  return (sizeof(K) + sizeof(u32)) * kSortTile;
}

// Runs the passes of a sort whose histograms are already in scratch.hist (zeroed scratch otherwise).
// Pass p reads buffer (p even ? 0 : 1) and writes the other one; returns true when the sorted
// result is in (k1, v1). iotaValues: the first pass generates values 0..n-1 instead of reading v0.
inline bool sort_staging_enabled()
{
  static const bool on = [] {
    const char* v = std::getenv("OTG_SORT_STAGE");
    return v && v[0] == '1';
  }();
  return on;
}

template<typename K>
inline bool onesweep_passes(K* k0, u32* v0, K* k1, u32* v1, u64 n, u32 shift0, u32 passes, bool iotaValues, SortScratch& s, u32* err, cudaStream_t st)
{
  const bool stage = sort_staging_enabled();
  auto kfn = stage ? onesweep_pass_kernel<K, false, false, true> : onesweep_pass_kernel<K>;
  cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(onesweep_smem_bytes<K>()));
  const u32 tiles = u32(SortScratch::tiles(n));
  if (passes)
    digit_base_kernel<<<passes, kRadix, 0, st>>>(s.hist);
  for (u32 p = 0; p < passes; ++p)
  {
    const bool even = (p % 2) == 0;
    const K* ki = even ? k0 : k1;
    const u32* vi = (p == 0 && iotaValues) ? nullptr : (even ? v0 : v1);
    K* ko = even ? k1 : k0;
    u32* vo = even ? v1 : v0;
    kfn<<<tiles, kSortThreads, onesweep_smem_bytes<K>(), st>>>(ki, vi, ko, vo, u32(n), shift0 + kRadixBits * p, s.hist + p * kRadix,
                                                               s.status + size_t(p) * tiles * kRadix, s.tileCounters + p, err, nullptr, nullptr);
  }
  return (passes % 2) == 1;
}

// Passes over a count known only on the device (*nDev <= n): launched for n elements.
template<typename K>
inline bool onesweep_passes_devn(K* k0, u32* v0, K* k1, u32* v1, u64 n, const unsigned long long* nDev, u32 shift0, u32 passes, bool iotaValues,
                                 SortScratch& s, u32* err, cudaStream_t st)
{
  cudaFuncSetAttribute(onesweep_pass_kernel<K, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(onesweep_smem_bytes<K>()));
  const u32 tiles = u32(SortScratch::tiles(n));
  if (passes)
    digit_base_kernel<<<passes, kRadix, 0, st>>>(s.hist);
  for (u32 p = 0; p < passes; ++p)
  {
    const bool even = (p % 2) == 0;
    const K* ki = even ? k0 : k1;
    const u32* vi = (p == 0 && iotaValues) ? nullptr : (even ? v0 : v1);
    K* ko = even ? k1 : k0;
    u32* vo = even ? v1 : v0;
    onesweep_pass_kernel<K, false, true><<<tiles, kSortThreads, onesweep_smem_bytes<K>(), st>>>(
      ki, vi, ko, vo, u32(n), shift0 + kRadixBits * p, s.hist + p * kRadix, s.status + size_t(p) * tiles * kRadix, s.tileCounters + p, err, nullptr,
      reinterpret_cast<const u64*>(nDev));
  }
  return (passes % 2) == 1;
}

// Segmented passes: `tiles` tiles listed in segTiles; hist holds [pass][segment][256] counts.
template<typename K>
inline bool onesweep_passes_segmented(K* k0, u32* v0, K* k1, u32* v1, u64 n, u32 passes, bool iotaValues, const uint2* segTiles, u32 tiles,
                                      const u64* segOff, u32 segments, u32* hist, u32* status, u32* counters, u32* err, cudaStream_t st)
{
  cudaFuncSetAttribute(onesweep_pass_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(onesweep_smem_bytes<K>()));
  if (tiles && passes && segments)
    digit_base_kernel<<<passes * segments, kRadix, 0, st>>>(hist);
  for (u32 p = 0; p < passes; ++p)
  {
    const bool even = (p % 2) == 0;
    const K* ki = even ? k0 : k1;
    const u32* vi = (p == 0 && iotaValues) ? nullptr : (even ? v0 : v1);
    K* ko = even ? k1 : k0;
    u32* vo = even ? v1 : v0;
    if (tiles)
      onesweep_pass_kernel<K, true><<<tiles, kSortThreads, onesweep_smem_bytes<K>(), st>>>(ki, vi, ko, vo, u32(n), kRadixBits * p,
                                                                                   hist + u64(p) * segments * kRadix, status + size_t(p) * tiles * kRadix,
                                                                                   counters + p, err, segTiles, segOff);
  }
  return (passes % 2) == 1;
}

} // namespace otg
