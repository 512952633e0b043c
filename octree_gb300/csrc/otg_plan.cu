// otg_plan.cu — one step of a forest workload recorded as a CUDA graph and replayed.
//
// A step is the forest Create of new entity values (same tree sizes) followed by batched
// RangeSearch, RayIntersectedAll and FrustumCulling over all trees. The first step runs through
// the ordinary calls (allocations, host-side sizing); it fixes every buffer, sizes the result
// buffers from its result counts (times a capacity factor) and is then recorded on a capture
// stream: the forest kernels, the batched query kernels appending into fixed-capacity buffers,
// and the result assembly, whose radix sorts and CSR offsets read the result counts from device
// memory. Replays launch that graph: no allocation, no host round trip inside the step. After a
// replay the host reads the counts once; a count above its capacity is reported as an error
// (the plan is then rebuilt with a larger factor).
#include "otg_query.cuh"

#include <new>

#include <cmath>
#include <memory>

namespace otg
{

// ---------------------------------------------------------------- result assembly, device counts
__device__ __forceinline__ u64 dev_count(const unsigned long long* m, u64 cap)
{
  return min(u64(*m), cap);
}

__global__ void plan_split_kernel(const u64* __restrict__ items, const unsigned long long* __restrict__ m, u64 cap, u32* __restrict__ qid,
                                  u32* __restrict__ ids)
{
  const u64 n = dev_count(m, cap);
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    const u64 it = items[i];
    qid[i] = u32(it >> 32);
    ids[i] = u32(it);
  }
}

// offsets[q] = first position of query q among the sorted query ids; offsets[nq] = count
__global__ void plan_offsets_kernel(const u32* __restrict__ qid, const unsigned long long* __restrict__ m, u64 cap, u64 nq, u64* __restrict__ offsets)
{
  const u64 n = dev_count(m, cap);
  for (u64 q = blockIdx.x * u64(blockDim.x) + threadIdx.x; q <= nq; q += u64(gridDim.x) * blockDim.x)
  {
    u64 lo = 0, hi = n;
    while (lo < hi)
    {
      const u64 mid = (lo + hi) >> 1;
      if (qid[mid] < q)
        lo = mid + 1;
      else
        hi = mid;
    }
    offsets[q] = q == nq ? n : lo;
  }
}

__global__ void plan_iota_ids_kernel(const u64* __restrict__ items, const unsigned long long* __restrict__ m, u64 cap, u32* __restrict__ perm,
                                     u32* __restrict__ key)
{
  const u64 n = dev_count(m, cap);
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    perm[i] = u32(i);
    key[i] = u32(items[i]);
  }
}

__global__ void plan_dist_bits_kernel(const double* __restrict__ d, const u32* __restrict__ perm, const unsigned long long* __restrict__ m, u64 cap,
                                      u64* __restrict__ key)
{
  const u64 n = dev_count(m, cap);
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
    key[i] = u64(__double_as_longlong(d[perm[i]])); // distances are non-negative
}

__global__ void plan_qid_kernel(const u64* __restrict__ items, const u32* __restrict__ perm, const unsigned long long* __restrict__ m, u64 cap,
                                u32* __restrict__ key)
{
  const u64 n = dev_count(m, cap);
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
    key[i] = u32(items[perm[i]] >> 32);
}

__global__ void plan_final_kernel(const u64* __restrict__ items, const double* __restrict__ d, const u32* __restrict__ perm,
                                  const unsigned long long* __restrict__ m, u64 cap, u32* __restrict__ ids, double* __restrict__ dist)
{
  const u64 n = dev_count(m, cap);
  for (u64 i = blockIdx.x * u64(blockDim.x) + threadIdx.x; i < n; i += u64(gridDim.x) * blockDim.x)
  {
    const u32 p = perm[i];
    ids[i] = u32(items[p]);
    dist[i] = d[p];
  }
}

// ---------------------------------------------------------------- plan state
enum PlanKind
{
  kPlanRange = 0,
  kPlanRayAll = 1,
  kPlanFrustum = 2
};

struct PlanQuery
{
  int kind = 0;
  const void* input = nullptr;
  u64 nq = 0;
  u32 np = 0;
  int mode = 0;
  u64 cap = 0;
  DevBuf qoff, qTree;
  DevBuf items, dist, count, err, work;
  DevBuf keysB, vals, valsB, perm, permB, k32, k32B, k64, k64B, scratch;
  DevBuf offsets, ids, rdist;
  const u32* idsOut = nullptr;
  const double* distOut = nullptr;
  u64 lastCount = 0;
};

struct Plan
{
  TreeState* t = nullptr;
  const void* ent = nullptr;
  double tol = -1.0;
  PlanQuery q[3];
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ran = false;
  ~Plan()
  {
    if (exec)
      cudaGraphExecDestroy(exec);
    if (graph)
      cudaGraphDestroy(graph);
    if (cap)
      cudaStreamDestroy(cap);
  }
};

static u32 bits_of(u64 v)
{
  u32 b = 0;
  while (v)
  {
    ++b;
    v >>= 1;
  }
  return b;
}

// sorts keys (device count) in place by `bits` bits, values alongside; returns the buffers that hold
// the result (the passes alternate between the two)
template<typename K>
static void plan_sort(K*& k, u32*& v, K*& kB, u32*& vB, u64 cap, const unsigned long long* m, u32 bits, DevBuf& scratch, u32* err, cudaStream_t st)
{
  const u32 passes = (bits + kRadixBits - 1) / kRadixBits;
  cudaMemsetAsync(scratch.p, 0, SortScratch::bytes(cap, passes), st);
  SortScratch ss;
  ss.carve(scratch.p, cap, passes);
  radix_histogram_kernel<K><<<blocks_for(cap), 256, 0, st>>>(k, cap, 0, passes, ss.hist, m);
  if (onesweep_passes_devn<K>(k, v, kB, vB, cap, m, 0, passes, false, ss, err, st))
  {
    std::swap(k, kB);
    std::swap(v, vB);
  }
}

template<typename T>
static int plan_record_query(Plan& p, PlanQuery& q, cudaStream_t st)
{
  TreeState& t = *p.t;
  TreeView<T> tv = view<T>(t, q.qTree.as<u32>());
  tv.nNodes = u32(t.maxNodes); // node counts vary between steps: bound by the allocation
  const T tl = tol_of<T>(p.tol);
  cudaMemsetAsync(q.count.p, 0, sizeof(unsigned long long), st);
  cudaMemsetAsync(q.err.p, 0, sizeof(u32), st);
  const bool withDist = q.kind == kPlanRayAll;
  Appender a{ q.items.as<u64>(), withDist ? q.dist.as<double>() : nullptr, q.count.as<unsigned long long>(), q.cap };
  // the warp shape the first (ordinary) run chose
  static const char* ops[3] = { "range", "ray all", "frustum" };
  const int shape = tune_lookup(query_key(ops[q.kind], OTG_ALGO_FILTERED, true, sizeof(T) == 8, t.kind, t.n, q.nq), 4);
  int rc;
  if (q.kind == kPlanRange)
    rc = batch_range<T>(tv, (const T*)q.input, u32(q.nq), q.mode, tl, a, q.work.as<u32>(), q.err.as<u32>(), st, shape, q.work.bytes);
  else if (q.kind == kPlanFrustum)
    rc = batch_frustum<T>(tv, (const T*)q.input, q.np, u32(q.nq), tl, a, q.work.as<u32>(), q.err.as<u32>(), st, shape, q.work.bytes);
  else
    rc = batch_ray_all<T>(tv, (const T*)q.input, u32(q.nq), tl, T(0), Lim<T>::max(), a, q.work.as<u32>(), q.err.as<u32>(), st, shape, q.work.bytes);
  if (rc)
    return rc;
  const unsigned long long* m = q.count.as<unsigned long long>();
  u32* err = q.err.as<u32>();
  const int blocks = blocks_for(q.cap);
  if (!withDist)
  {
    u64* k = q.items.as<u64>();
    u64* kB = q.keysB.as<u64>();
    u32* v = q.vals.as<u32>();
    u32* vB = q.valsB.as<u32>();
    plan_sort<u64>(k, v, kB, vB, q.cap, m, 32 + bits_of(q.nq), q.scratch, err, st);
    plan_split_kernel<<<blocks, 256, 0, st>>>(k, m, q.cap, q.k32.as<u32>(), q.ids.as<u32>());
    plan_offsets_kernel<<<blocks_for(q.nq + 1), 256, 0, st>>>(q.k32.as<u32>(), m, q.cap, q.nq, q.offsets.as<u64>());
    q.idsOut = q.ids.as<u32>();
    q.distOut = nullptr;
  }
  else
  {
    u32* perm = q.perm.as<u32>();
    u32* permB = q.permB.as<u32>();
    u32* k32 = q.k32.as<u32>();
    u32* k32B = q.k32B.as<u32>();
    u64* k64 = q.k64.as<u64>();
    u64* k64B = q.k64B.as<u64>();
    plan_iota_ids_kernel<<<blocks, 256, 0, st>>>(q.items.as<u64>(), m, q.cap, perm, k32);
    plan_sort<u32>(k32, perm, k32B, permB, q.cap, m, bits_of(t.n), q.scratch, err, st);
    plan_dist_bits_kernel<<<blocks, 256, 0, st>>>(q.dist.as<double>(), perm, m, q.cap, k64);
    plan_sort<u64>(k64, perm, k64B, permB, q.cap, m, 64, q.scratch, err, st);
    plan_qid_kernel<<<blocks, 256, 0, st>>>(q.items.as<u64>(), perm, m, q.cap, k32);
    plan_sort<u32>(k32, perm, k32B, permB, q.cap, m, bits_of(q.nq), q.scratch, err, st);
    plan_final_kernel<<<blocks, 256, 0, st>>>(q.items.as<u64>(), q.dist.as<double>(), perm, m, q.cap, q.ids.as<u32>(), q.rdist.as<double>());
    plan_offsets_kernel<<<blocks_for(q.nq + 1), 256, 0, st>>>(k32, m, q.cap, q.nq, q.offsets.as<u64>());
    q.idsOut = q.ids.as<u32>();
    q.distOut = q.rdist.as<double>();
  }
  return cuda_status(cudaGetLastError(), "recording a query");
}

static int plan_alloc(PlanQuery& q, u64 nEntities)
{
  const u64 cap = q.cap;
  const u32 bitsMax = 64;
  const u32 passes = (bitsMax + kRadixBits - 1) / kRadixBits;
  cudaError_t e;
  if ((e = q.items.ensure(sizeof(u64) * cap)) || (e = q.count.ensure(sizeof(unsigned long long))) || (e = q.err.ensure(sizeof(u32))) ||
      (e = q.work.ensure(batch_work_bytes(q.nq))) || (e = q.keysB.ensure(sizeof(u64) * cap)) || (e = q.vals.ensure(sizeof(u32) * cap)) ||
      (e = q.valsB.ensure(sizeof(u32) * cap)) || (e = q.k32.ensure(sizeof(u32) * cap)) || (e = q.scratch.ensure(SortScratch::bytes(cap, passes))) ||
      (e = q.offsets.ensure(sizeof(u64) * (q.nq + 1))) || (e = q.ids.ensure(sizeof(u32) * cap)))
    return cuda_status(e, "allocating plan buffers");
  if (q.kind == kPlanRayAll)
    if ((e = q.dist.ensure(sizeof(double) * cap)) || (e = q.perm.ensure(sizeof(u32) * cap)) || (e = q.permB.ensure(sizeof(u32) * cap)) ||
        (e = q.k32B.ensure(sizeof(u32) * cap)) || (e = q.k64.ensure(sizeof(u64) * cap)) || (e = q.k64B.ensure(sizeof(u64) * cap)) ||
        (e = q.rdist.ensure(sizeof(double) * cap)))
      return cuda_status(e, "allocating plan buffers");
  (void)nEntities;
  return OTG_OK;
}

int plan_create(Plan& p, TreeState& t, const void* ent, const u64* treeOff, u32 trees, u32 maxDepth, u64 maxElem, const void* inputs[3],
                const u64* qoff[3], u32 np, int mode, double tol, double capScale, cudaStream_t st)
{
  p.t = &t;
  p.ent = ent;
  p.tol = tol;
  // 1. an ordinary step: the forest, the queries, their result sizes
  if (int rc = build_forest(t, ent, treeOff, trees, maxDepth, nullptr, maxElem, OTG_MEM_DEVICE, st))
    return rc;
  if (int rc = finish_build(t, st))
    return rc;
  for (int k = 0; k < 3; ++k)
  {
    PlanQuery& q = p.q[k];
    q.kind = k;
    q.input = inputs[k];
    q.np = np;
    q.mode = mode;
    if (!qoff[k] || !inputs[k])
      continue;
    if (int rc = forest_query_trees(t, qoff[k], q.qoff, q.qTree, q.nq, st))
      return rc;
    if (q.nq == 0)
      continue;
    ResultState r;
    int rc;
    if (k == kPlanRange)
      rc = query_range(t, q.input, q.nq, mode, tol, OTG_ALGO_FILTERED, r, OTG_MEM_DEVICE, st, q.qTree.as<u32>());
    else if (k == kPlanRayAll)
      rc = query_ray(t, q.input, q.nq, tol, 0.0, -1.0, false, OTG_ALGO_FILTERED, r, OTG_MEM_DEVICE, st, q.qTree.as<u32>());
    else
      rc = query_frustum(t, q.input, np, q.nq, tol, OTG_ALGO_FILTERED, r, OTG_MEM_DEVICE, st, q.qTree.as<u32>());
    if (rc)
      return rc;
    q.cap = std::max<u64>(4096, u64(std::ceil(double(r.nids) * std::max(1.0, capScale))));
    if (int rc2 = plan_alloc(q, t.n))
      return rc2;
  }
  // 2. record the step
  cudaError_t e = cudaStreamCreateWithFlags(&p.cap, cudaStreamNonBlocking);
  if (!e)
    e = cudaStreamBeginCapture(p.cap, cudaStreamCaptureModeThreadLocal);
  if (e)
    return cuda_status(e, "starting the graph capture");
  int rc = forest_relaunch(t, ent, nullptr, p.cap);
  for (int k = 0; k < 3 && !rc; ++k)
    if (p.q[k].nq)
      rc = t.scalar == OTG_SCALAR_F64 ? plan_record_query<double>(p, p.q[k], p.cap) : plan_record_query<float>(p, p.q[k], p.cap);
  e = cudaStreamEndCapture(p.cap, &p.graph);
  if (rc)
    return rc;
  if (e)
    return cuda_status(e, "ending the graph capture");
  if ((e = cudaGraphInstantiate(&p.exec, p.graph, 0)))
    return cuda_status(e, "instantiating the graph");
  return OTG_OK;
}

int plan_run(Plan& p, cudaStream_t st)
{
  p.ran = true;
  return cuda_status(cudaGraphLaunch(p.exec, st), "launching the recorded step");
}

int plan_result(Plan& p, int which, cudaStream_t st, u64& nq, u64& nids, const u64*& offsets, const u32*& ids, const double*& dist)
{
  if (which < 0 || which > 2 || !p.ran)
  {
    set_error("plan result: which must be 0, 1 or 2, after a run");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  PlanQuery& q = p.q[which];
  unsigned long long c = 0;
  u32 err = 0;
  cudaError_t e = cudaSuccess;
  if (q.nq)
  {
    e = cudaMemcpyAsync(&c, q.count.p, sizeof(c), cudaMemcpyDeviceToHost, st);
    if (!e)
      e = cudaMemcpyAsync(&err, q.err.p, sizeof(err), cudaMemcpyDeviceToHost, st);
  }
  u32 buildErr = 0;
  if (!e)
    e = cudaMemcpyAsync(&buildErr, p.t->err.p, sizeof(buildErr), cudaMemcpyDeviceToHost, st);
  if (!e)
    e = cudaStreamSynchronize(st);
  if (e)
    return cuda_status(e, "reading the step's result");
  if ((err | buildErr) & kErrTimeout)
  {
    set_error("a bounded device wait ran out");
    return OTG_ERR_TIMEOUT;
  }
  if (buildErr & kErrCapacity)
  {
    set_error("node capacity exceeded during emission");
    return OTG_ERR_OUT_OF_MEMORY;
  }
  if (err & kErrStack)
  {
    set_error("traversal stack bound exceeded");
    return OTG_ERR_NOT_SUPPORTED;
  }
  if (c > q.cap)
  {
    set_error("the step's results exceed the plan's capacity: create the plan with a larger capacity factor");
    return OTG_ERR_OUT_OF_MEMORY;
  }
  nq = q.nq;
  nids = c;
  offsets = q.nq ? q.offsets.as<u64>() : nullptr;
  ids = q.idsOut;
  dist = q.distOut;
  return OTG_OK;
}

} // namespace otg

using namespace otg;

struct otg_plan
{
  otg::Plan p;
};


extern "C" int otg_forest_plan_new(otg_plan** out, otg_tree* tree, const void* entities, const uint64_t* tree_offsets, uint32_t n_trees, uint32_t max_depth,
                        uint64_t max_elements, const void* ranges, const uint64_t* range_offsets, int mode, const void* rays, const uint64_t* ray_offsets,
                        const void* planes, uint64_t planes_per_query, const uint64_t* frustum_offsets, double tol, double capacity_factor,
                        void* stream)
{
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
  {
    cudaGetLastError();
    set_error("no CUDA device is available; this library has no CPU path");
    return OTG_ERR_NO_DEVICE;
  }
  if (!out || !tree || !entities || !tree_offsets || (mode != OTG_RANGE_INSIDE && mode != OTG_RANGE_OVERLAP) || (planes && planes_per_query == 0))
  {
    set_error("otg_forest_plan_new: invalid argument");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  auto* p = new (std::nothrow) otg_plan();
  if (!p)
    return OTG_ERR_OUT_OF_MEMORY;
  const void* inputs[3] = { ranges, rays, planes };
  const u64* qoff[3] = { range_offsets, ray_offsets, frustum_offsets };
  int rc = plan_create(p->p, tree->s, entities, tree_offsets, n_trees, max_depth, max_elements, inputs, qoff,
                       u32(planes_per_query), mode, tol, capacity_factor, (cudaStream_t)stream);
  if (rc)
  {
    delete p;
    *out = nullptr;
    return rc;
  }
  *out = p;
  return OTG_OK;
}

extern "C" int otg_forest_plan_run(otg_plan* plan, void* stream)
{
  if (!plan)
    return OTG_ERR_INVALID_ARGUMENT;
  return plan_run(plan->p, (cudaStream_t)stream);
}

extern "C" int otg_forest_plan_result(otg_plan* plan, int which, uint64_t* n_queries, uint64_t* n_ids, const uint64_t** offsets, const uint32_t** ids,
                           const double** distances, void* stream)
{
  if (!plan || !n_queries || !n_ids || !offsets || !ids)
    return OTG_ERR_INVALID_ARGUMENT;
  u64 nq = 0, nids = 0;
  const u64* o = nullptr;
  const u32* i = nullptr;
  const double* d = nullptr;
  int rc = plan_result(plan->p, which, (cudaStream_t)stream, nq, nids, o, i, d);
  if (rc)
    return rc;
  *n_queries = nq;
  *n_ids = nids;
  *offsets = o;
  *ids = i;
  if (distances)
    *distances = d;
  return OTG_OK;
}

extern "C" void otg_forest_plan_free(otg_plan* plan) { delete plan; }

/* copies the last run's result `which` into caller arrays (mem: destination space) */
extern "C" int otg_forest_plan_copy(otg_plan* plan, int which, uint64_t* offsets, uint32_t* ids, double* distances, int mem, void* stream)
{
  u64 nq = 0, nids = 0;
  const u64* o = nullptr;
  const u32* i = nullptr;
  const double* d = nullptr;
  if (!plan)
    return OTG_ERR_INVALID_ARGUMENT;
  if (int rc = plan_result(plan->p, which, (cudaStream_t)stream, nq, nids, o, i, d))
    return rc;
  const cudaMemcpyKind kind = mem == OTG_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  cudaError_t e = cudaSuccess;
  if (nq && offsets)
    e = cudaMemcpyAsync(offsets, o, sizeof(u64) * (nq + 1), kind, (cudaStream_t)stream);
  if (!e && nids && ids)
    e = cudaMemcpyAsync(ids, i, sizeof(u32) * nids, kind, (cudaStream_t)stream);
  if (!e && nids && distances && d)
    e = cudaMemcpyAsync(distances, d, sizeof(double) * nids, kind, (cudaStream_t)stream);
  if (!e)
    e = cudaStreamSynchronize((cudaStream_t)stream);
  return cuda_status(e, "copying the step's result");
}
