// otg_tune.cu — kernel-shape autotuner.
//
// Several kernels exist in interchangeable shapes that return identical results: one query per
// thread or one query per warp, and 2, 4 or 8 warps per block for the persistent warp kernels.
// Which one is fastest depends on the tree and the batch (entities per node, query count and
// extent). The first call of a kernel on a size class (kind, scalar, log2 of the entity count,
// log2 of the query count) times every candidate shape on that call's own work with CUDA events,
// keeps the fastest for the class and returns the result of a final run with it; later calls of
// the class run the kept shape directly.
#include "otg_internal.h"

#include <cstdio>
#include <map>
#include <mutex>

namespace otg
{

struct TuneEntry
{
  std::string key;
  int best = 0;
  std::string bestName;
  std::vector<std::pair<std::string, float>> timings;
};

struct Tuner
{
  std::mutex m;
  bool enabled = true;
  int forced = -1; // a shape every call that offers it runs (diagnostics)
  std::map<std::string, size_t> index;
  std::vector<TuneEntry> entries;
};

static Tuner& tuner()
{
  static Tuner t;
  return t;
}

static u32 log2_bucket(u64 v)
{
  u32 b = 0;
  while (v > 1)
  {
    v >>= 1;
    ++b;
  }
  return b;
}

std::string tune_key(const char* op, bool f64, int kind, u64 entities, u64 queries)
{
  char buf[128];
  std::snprintf(buf, sizeof(buf), "%s %s %s n=2^%u q=2^%u", op, f64 ? "f64" : "f32", kind != OTG_KIND_POINTS ? "boxes" : "points", log2_bucket(entities),
                log2_bucket(queries));
  return buf;
}

int tune_run(const std::string& key, const std::vector<std::pair<int, const char*>>& cands, int fallback, cudaStream_t st,
             const std::function<int(int)>& launch)
{
  Tuner& T = tuner();
  {
    std::lock_guard<std::mutex> g(T.m);
    if (T.forced >= 0)
      for (const auto& c : cands)
        if (c.first == T.forced)
          return launch(T.forced);
    if (!T.enabled || cands.size() < 2)
      return launch(cands.size() == 1 ? cands[0].first : fallback);
    auto it = T.index.find(key);
    if (it != T.index.end())
    {
      const int best = T.entries[it->second].best;
      return launch(best);
    }
  }
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (!e)
    e = cudaEventCreate(&b);
  if (e)
  {
    if (a)
      cudaEventDestroy(a);
    return cuda_status(e, "creating tuning events");
  }
  TuneEntry entry;
  entry.key = key;
  float bestMs = 0.f;
  int best = fallback;
  int rc = OTG_OK;
  for (const auto& c : cands)
  {
    cudaEventRecord(a, st);
    rc = launch(c.first);
    cudaEventRecord(b, st);
    if (rc)
      break;
    if ((e = cudaEventSynchronize(b)))
    {
      rc = cuda_status(e, "timing a kernel shape");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    entry.timings.emplace_back(c.second, ms);
    if (entry.timings.size() == 1 || ms < bestMs)
    {
      bestMs = ms;
      best = c.first;
      entry.bestName = c.second;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc)
    return rc;
  entry.best = best;
  {
    std::lock_guard<std::mutex> g(T.m);
    if (!T.index.count(key))
    {
      T.index[key] = T.entries.size();
      T.entries.push_back(entry);
    }
  }
  return launch(best);
}

int tune_lookup(const std::string& key, int fallback)
{
  std::lock_guard<std::mutex> g(tuner().m);
  auto it = tuner().index.find(key);
  return it == tuner().index.end() ? fallback : tuner().entries[it->second].best;
}

void tune_force(int shape)
{
  std::lock_guard<std::mutex> g(tuner().m);
  tuner().forced = shape;
}

void tune_enable(bool on)
{
  std::lock_guard<std::mutex> g(tuner().m);
  tuner().enabled = on;
}

int tune_count()
{
  std::lock_guard<std::mutex> g(tuner().m);
  return int(tuner().entries.size());
}

std::string tune_entry(int i)
{
  std::lock_guard<std::mutex> g(tuner().m);
  Tuner& T = tuner();
  if (i < 0 || size_t(i) >= T.entries.size())
    return {};
  const TuneEntry& en = T.entries[size_t(i)];
  std::string s = en.key + ":";
  for (const auto& t : en.timings)
  {
    char buf[64];
    std::snprintf(buf, sizeof(buf), " %s %.3f ms", t.first.c_str(), t.second);
    s += buf;
  }
  s += " -> " + en.bestName;
  return s;
}

} // namespace otg
