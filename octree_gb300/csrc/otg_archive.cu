// otg_archive.cu — a built tree as the reference's binary archive of its static tree, and a tree
// resumed from such an archive (host code).
//
// The bytes are those BinaryOutputArchive (serialization/binary_archive.h) writes for
// `ar & tree` with tree a StaticOctreePoint / StaticOctreeBox, or their Managed forms
// StaticOctreePointM / StaticOctreeBoxM that also hold the entities:
//   StaticLinearOrthoTreeCore (serialization.h:373-385): u32 version, then its base
//   OrthoTreeCoreBase (:359-370): u32 version, u64 maxElementNum, u32 maxDepthID, the nominal
//   tree box {minPoint, size} (MBR trees only), the node size table (MinPoint trees only);
//   then the node storage variant (u32 index + NodeStorage256 / 65536 / General: child segment
//   begins, {begin, length} entity segments), the depth ids, the entity storage and the node
//   geometry; the Managed form appends the entities (:433-438).
// Scalars are written raw in little-endian order; every vector and every std::array starts with
// a u32 size tag (serialized_size_t without ORTHOTREE__LARGE_DATASET, core/types.h:51-55;
// serialization/stl/vector.h, array.h, variant.h; std::monostate writes nothing, stl/common.h).
// The node storage is the narrowest that IsFit allows for GetMaxPossibleNodeCount
// (core/ot_static_linear_core.h:326-344, :370-376, :574-580).
#include "otg_internal.h"

#include <cstring>
#include <limits>

static_assert(__BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__, "the archive is little-endian and written as the host stores scalars");

namespace otg
{
namespace
{

struct ArchiveOut
{
  std::vector<unsigned char> bytes;
  template<typename V>
  void put(V v)
  {
    unsigned char b[sizeof(V)];
    std::memcpy(b, &v, sizeof(V));
    bytes.insert(bytes.end(), b, b + sizeof(V));
  }
  void tag(u64 n) { put(u32(n)); }
  template<typename T>
  void vec3(const T* v)
  {
    tag(3);
    for (int c = 0; c < 3; ++c)
      put(v[c]);
  }
};

struct ArchiveIn
{
  const unsigned char* p;
  u64 size, pos = 0;
  bool ok = true;
  template<typename V>
  V get()
  {
    V v{};
    if (!ok || size - pos < sizeof(V))
    {
      ok = false;
      return v;
    }
    std::memcpy(&v, p + pos, sizeof(V));
    pos += sizeof(V);
    return v;
  }
  // a size tag that must be followed by at least `n * minBytes` bytes
  u64 tag(u64 minBytes)
  {
    const u64 n = get<u32>();
    if (ok && minBytes && n > (size - pos) / minBytes)
      ok = false;
    return ok ? n : 0;
  }
  template<typename T>
  void vec3(T* v)
  {
    if (tag(sizeof(T)) != 3)
      ok = false;
    for (int c = 0; c < 3; ++c)
      v[c] = get<T>();
  }
};

// GetMaxPossibleNodeCount (core/ot_static_linear_core.h:326-344) for 3-D trees
u64 max_possible_node_count(u64 n, u32 D)
{
  auto nodeNum = [](u32 d) { return ((u64(1) << (3 * d)) - 1) / 7; };
  const u64 byDepth = nodeNum(D);
  u32 bw = 0;
  for (u64 v = n - 1; v; v >>= 1)
    ++bw;
  const u32 full = std::min<u32>(D, bw / 3);
  const u64 byEntities = nodeNum(full) + u64(D - full) * n;
  return std::min(byEntities, byDepth);
}

// the node storage variant index Create picks (:574-580 with IsFit, :370-376)
u32 storage_index(u64 n, u32 D)
{
  if (n == 0)
    return 0; // Create of no entities returns before choosing: the default alternative
  const u64 m = max_possible_node_count(n, D);
  if (m < 0xffu && n < 0xffu)
    return 0;
  if (m < 0xffffu && n < 0xffffu)
    return 1;
  return 2;
}

template<typename W>
void put_storage(ArchiveOut& a, const std::vector<u32>& childBegins, const std::vector<u32>& seg)
{
  a.tag(childBegins.size());
  for (u32 v : childBegins)
    a.put(W(v));
  a.tag(seg.size() / 2);
  for (u32 v : seg)
    a.put(W(v));
}

} // namespace

namespace
{

// Host copies of everything the archive holds, from the tree's static layout.
template<typename T>
struct StaticHost
{
  std::vector<u32> childBegins, seg, storage;
  std::vector<unsigned char> depth;
  std::vector<T> geometry, entities;
  Space<T> sp{};
};

template<typename T>
int gather_static(TreeState& t, bool managed, StaticHost<T>& h, cudaStream_t st)
{
  otg_static_layout L;
  if (int rc = export_static(t, &L, st))
    return rc;
  const u64 m = L.node_count, n = t.n;
  const size_t W = t.kind == OTG_KIND_POINTS ? 3 : 6;
  h.childBegins.resize(L.child_begin_count);
  h.seg.resize(2 * m);
  h.depth.resize(m);
  h.storage.resize(n);
  h.geometry.resize(m * L.geometry_per_node);
  // the entities in input order come from the tree's own sorted copy (entity storage[i] is the
  // id of sortedGeom[i]): a tree built from device memory holds no input-order copy of them
  std::vector<T> sorted(managed ? n * W : 0);
  struct Part
  {
    void* dst;
    const void* src;
    size_t bytes;
  } parts[] = { { h.childBegins.data(), L.child_begins, sizeof(u32) * h.childBegins.size() },
                { h.seg.data(), L.entity_segments, sizeof(u32) * h.seg.size() },
                { h.depth.data(), L.depth_ids, h.depth.size() },
                { h.storage.data(), L.entity_storage, sizeof(u32) * h.storage.size() },
                { h.geometry.data(), L.geometry, sizeof(T) * h.geometry.size() },
                { sorted.data(), t.sortedGeom.p, sizeof(T) * sorted.size() },
                { &h.sp, t.space.p, (n && t.space.p) ? sizeof(Space<T>) : 0 } };
  for (const Part& p : parts)
    if (p.bytes)
      if (cudaError_t e = cudaMemcpy(p.dst, p.src, p.bytes, cudaMemcpyDeviceToHost))
        return cuda_status(e, "copying the tree for its archive");
  if (n == 0)
  {
    // a build of no entities computes no space: Create still runs InitBase on the given box, or on
    // the bounding box of nothing (inverted: min = +max, max = -max, so the size overflows)
    T box[6];
    if (t.boxGiven && t.boxDev.p)
    {
      if (cudaError_t e = cudaMemcpy(box, t.boxDev.p, sizeof(box), cudaMemcpyDeviceToHost))
        return cuda_status(e, "copying the space box");
    }
    else
      for (int d = 0; d < 3; ++d)
      {
        box[d] = std::numeric_limits<T>::max();
        box[3 + d] = -std::numeric_limits<T>::max();
      }
    for (int d = 0; d < 3; ++d)
    {
      h.sp.min[d] = box[d];
      h.sp.max[d] = box[3 + d];
      h.sp.size[d] = T(box[3 + d] - box[d]);
    }
  }
  if (managed)
  {
    h.entities.resize(n * W);
    for (u64 i = 0; i < n; ++i)
    {
      const u32 id = h.storage[i];
      if (id >= n)
      {
        set_error("archive: entity storage holds an id out of range");
        return OTG_ERR_CUDA;
      }
      std::memcpy(&h.entities[size_t(id) * W], &sorted[i * W], sizeof(T) * W);
    }
  }
  return OTG_OK;
}

// The archive of the tree's static layout (core only, or with the entities). esBegin / esEnd: the
// byte range of the entity storage section.
template<typename T>
void write_archive(const TreeState& t, const StaticHost<T>& h, bool managed, ArchiveOut& a, u64& esBegin, u64& esEnd)
{
  const bool box = t.kind != OTG_KIND_POINTS;
  const size_t vec = 4 + 3 * sizeof(T), groups = box ? 2 : 1;
  a.bytes.reserve(64 + (t.D + 2) * vec + h.depth.size() * (9 + groups * vec) + t.n * (4 + (managed ? groups * vec : 0)));
  a.put(u32(0)); // StaticLinearOrthoTreeCore SERIALIZED_VERSION_ID
  a.put(u32(0)); // OrthoTreeCoreBase SERIALIZED_VERSION_ID
  a.put(u64(t.maxElem));
  a.put(u32(t.D));
  if (box)
  {
    a.vec3(h.sp.min); // m_nominalTreeBox {minPoint, size}
    a.vec3(h.sp.size);
  }
  else
  {
    // m_nodeSize of InitBase (core/ot_base.h:121-134): depth 0 .. D + 1, size halved per depth
    a.tag(t.D + 2);
    T lf = T(1);
    for (u32 d = 0; d < t.D + 2; ++d, lf *= T(0.5))
    {
      const T v[3] = { h.sp.size[0] * lf, h.sp.size[1] * lf, h.sp.size[2] * lf };
      a.vec3(v);
    }
  }
  const u32 idx = storage_index(t.n, t.D);
  a.put(idx);
  if (idx == 0)
    put_storage<uint8_t>(a, h.childBegins, h.seg);
  else if (idx == 1)
    put_storage<uint16_t>(a, h.childBegins, h.seg);
  else
    put_storage<uint32_t>(a, h.childBegins, h.seg);
  a.tag(h.depth.size());
  for (unsigned char d : h.depth)
    a.put(d);
  esBegin = a.bytes.size();
  a.tag(h.storage.size());
  for (u32 id : h.storage)
    a.put(id);
  esEnd = a.bytes.size();
  const size_t gw = box ? 6 : 3;
  a.tag(h.depth.size());
  for (size_t i = 0; i < h.depth.size(); ++i)
  {
    a.vec3(&h.geometry[i * gw]);
    if (box)
      a.vec3(&h.geometry[i * gw + 3]);
  }
  if (managed)
  {
    a.tag(t.n);
    for (u64 i = 0; i < t.n; ++i)
    {
      a.vec3(&h.entities[i * gw]);
      if (box)
        a.vec3(&h.entities[i * gw + 3]);
    }
  }
}

template<typename T>
int save_impl(TreeState& t, bool managed, std::vector<unsigned char>& out, cudaStream_t st)
{
  StaticHost<T> h;
  if (int rc = gather_static(t, managed, h, st))
    return rc;
  ArchiveOut a;
  u64 esBegin, esEnd;
  write_archive(t, h, managed, a, esBegin, esEnd);
  out = std::move(a.bytes);
  return OTG_OK;
}

template<typename T>
int load_impl(TreeState& t, const unsigned char* p, u64 size, const void* box, cudaStream_t st)
{
  const bool isBox = t.kind != OTG_KIND_POINTS;
  const size_t gw = isBox ? 6 : 3;
  const u64 vecBytes = 4 + 3 * sizeof(T);
  ArchiveIn in{ p, size };
  const u32 vCore = in.get<u32>(), vBase = in.get<u32>();
  const u64 maxElem = in.get<u64>();
  const u32 D = in.get<u32>();
  T tmp[3];
  if (isBox)
  {
    in.vec3(tmp);
    in.vec3(tmp);
  }
  else
  {
    const u64 cnt = in.tag(vecBytes);
    for (u64 i = 0; i < cnt && in.ok; ++i)
      in.vec3(tmp);
  }
  const u32 idx = in.get<u32>();
  const u32 width = idx == 0 ? 1u : idx == 1 ? 2u : 4u;
  auto skip = [&](u64 count, u64 each) {
    if (in.ok && count <= (in.size - in.pos) / each)
      in.pos += count * each;
    else
      in.ok = false;
  };
  skip(in.tag(width), width);                     // child segment begins
  skip(in.tag(2 * width), 2 * width);             // entity segments
  const u64 m = in.tag(1);
  skip(m, 1);                                     // depth ids
  skip(in.tag(4), 4);                             // entity storage
  const u64 mg = in.tag(gw / 3 * vecBytes);
  skip(mg, gw / 3 * vecBytes);                    // node geometry
  const u64 coreEnd = in.pos;
  if (!in.ok || vCore != 0 || vBase != 0 || idx > 2 || mg != m)
  {
    set_error("otg_tree_load_static: not a binary archive of this static tree type (or an unsupported version)");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (coreEnd == size)
  {
    set_error("otg_tree_load_static: the archive holds no entities; resuming needs the Managed form (StaticOctreePointM / StaticOctreeBoxM)");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  const u64 n = in.tag(gw / 3 * vecBytes);
  std::vector<T> ent(n * gw);
  for (u64 i = 0; i < n && in.ok; ++i)
  {
    in.vec3(&ent[i * gw]);
    if (isBox)
      in.vec3(&ent[i * gw + 3]);
  }
  if (!in.ok || in.pos != size || D < 1 || maxElem < 1)
  {
    set_error("otg_tree_load_static: malformed entity section, trailing bytes or invalid tree parameters");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  if (int rc = build_tree(t, ent.data(), n, D, box, maxElem, OTG_MEM_HOST, st))
    return rc;
  if (int rc = finish_build(t, st))
    return rc;
  // the rebuild must be the archived tree: every section equal, the entity storage equal per
  // node as a set (the reference's unstable sort orders equal locations arbitrarily)
  StaticHost<T> h;
  if (int rc = gather_static(t, false, h, st))
    return rc;
  ArchiveOut a;
  u64 esBegin, esEnd;
  write_archive(t, h, false, a, esBegin, esEnd);
  bool same = a.bytes.size() == coreEnd && std::memcmp(a.bytes.data(), p, esBegin) == 0 &&
              std::memcmp(a.bytes.data() + esEnd, p + esEnd, coreEnd - esEnd) == 0;
  if (same)
  {
    std::vector<u32> archived(n);
    std::memcpy(archived.data(), p + esBegin + 4, sizeof(u32) * n);
    for (size_t i = 0; same && 2 * i < h.seg.size(); ++i)
    {
      const u32 b = h.seg[2 * i], len = h.seg[2 * i + 1];
      std::vector<u32> x(archived.begin() + b, archived.begin() + b + len), y(h.storage.begin() + b, h.storage.begin() + b + len);
      std::sort(x.begin(), x.end());
      std::sort(y.begin(), y.end());
      same = x == y;
    }
  }
  if (!same)
  {
    set_error("otg_tree_load_static: rebuilding the archived entities does not give the archived tree (was it created with another space box?)");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  return OTG_OK;
}

} // namespace

int save_static_archive(TreeState& t, bool managed, void* buffer, u64 capacity, u64* size, cudaStream_t st)
{
  std::vector<unsigned char> bytes;
  const int rc = t.scalar == OTG_SCALAR_F64 ? save_impl<double>(t, managed, bytes, st) : save_impl<float>(t, managed, bytes, st);
  if (rc)
    return rc;
  *size = bytes.size();
  if (!buffer)
    return OTG_OK;
  if (capacity < bytes.size())
  {
    set_error("otg_tree_save_static: the buffer is smaller than the archive (its size is in *size)");
    return OTG_ERR_INVALID_ARGUMENT;
  }
  std::memcpy(buffer, bytes.data(), bytes.size());
  return OTG_OK;
}

int load_static_archive(TreeState& t, const void* buffer, u64 size, const void* box, cudaStream_t st)
{
  const auto* p = static_cast<const unsigned char*>(buffer);
  return t.scalar == OTG_SCALAR_F64 ? load_impl<double>(t, p, size, box, st) : load_impl<float>(t, p, size, box, st);
}

} // namespace otg
