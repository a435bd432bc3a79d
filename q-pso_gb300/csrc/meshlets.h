// meshlets.h -- host-side partition of a triangle mesh into meshlets for
// the fused kernels (plain C++, no CUDA).
#pragma once

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace qpso {

// Meshlet: up to kMletFaces faces whose corners reference at most kMletVerts
// unique vertices.  Payload at `off` bytes into the mesh's meshlet blob:
// nv float4 positions (x, y, z, 0; metres), then nf uint32 faces packing the
// three local vertex ids in bits 0-9, 10-19, 20-29, padded to 16 bytes.
// Built once at mesh upload; face order does not affect any result (depth
// writes are atomic minima, the render AABB is a min/max).  After the last
// payload the blob holds one object-space box per meshlet, two float4 (lo,
// hi) at `box_off`, over the meshlet's vertices: the fused kernels project
// its corners to skip meshlets that miss a tile band.  After them come the
// group boxes, the union of each run of kMletGroup meshlets' boxes, with
// which a culled pass of a large mesh skips whole groups.
constexpr int kMletFaces = 128;  // largest meshlet: faces
constexpr int kMletVerts = 128;  // largest meshlet: unique vertices (vertex cache slots)
constexpr int kMletBytes = kMletVerts * 16 + kMletFaces * 4;
constexpr int kMletGroup = 16;   // meshlets per group box
// Meshlet size by mesh size: meshes of up to kSmallMeshFaces faces are cut
// into meshlets of 64 faces / 64 vertices (finer work items balance a
// render over more warps, and a launch whose meshes are all small gets
// 1 KB vertex caches per warp); larger meshes into 128 / 128, whose fewer
// shared vertices and items cost less per face.
constexpr uint32_t kSmallMeshFaces = 16384;
inline int meshlet_cap(uint32_t num_faces) { return num_faces <= kSmallMeshFaces ? 64 : 128; }
struct MeshletHdr {
  uint32_t off;
  uint16_t nv;
  uint16_t nf;
};

inline size_t mlet_align16(size_t x) { return (x + 15) / 16 * 16; }

// Partition the faces into meshlets (`cap` faces and `cap` unique vertices
// at most, cap <= kMletFaces): vertices are deduplicated by exact bit pattern, then
// faces are grown breadth-first over shared vertices so that each meshlet
// is a compact surface patch whose vertices are transformed once per pose.
inline void build_meshlets(const float* soa, uint32_t F, std::vector<MeshletHdr>& hdr,
                           std::vector<unsigned char>& blob, size_t* box_off, int cap = kMletFaces) {
  struct Key {
    uint32_t x, y, z;
    bool operator==(const Key& o) const { return x == o.x && y == o.y && z == o.z; }
  };
  struct KeyHash {
    size_t operator()(const Key& k) const {
      uint64_t h = k.x * 0x9E3779B97F4A7C15ull;
      h ^= (h >> 29) + k.y * 0xBF58476D1CE4E5B9ull;
      h ^= (h >> 31) + k.z * 0x94D049BB133111EBull;
      return (size_t)(h ^ (h >> 32));
    }
  };
  std::unordered_map<Key, uint32_t, KeyHash> ids;
  ids.reserve(2 * (size_t)F);
  std::vector<float> pos;  // unique vertex positions
  std::vector<uint32_t> fv(3 * (size_t)F);
  for (uint32_t f = 0; f < F; ++f)
    for (int j = 0; j < 3; ++j) {
      float v[3] = {soa[f + (size_t)j * F], soa[f + (size_t)(3 + j) * F], soa[f + (size_t)(6 + j) * F]};
      Key k;
      std::memcpy(&k.x, &v[0], 4);
      std::memcpy(&k.y, &v[1], 4);
      std::memcpy(&k.z, &v[2], 4);
      auto it = ids.find(k);
      uint32_t id;
      if (it == ids.end()) {
        id = (uint32_t)(pos.size() / 3);
        ids.emplace(k, id);
        pos.insert(pos.end(), v, v + 3);
      } else {
        id = it->second;
      }
      fv[3 * (size_t)f + j] = id;
    }
  const uint32_t V = (uint32_t)(pos.size() / 3);
  // vertex -> faces (CSR)
  std::vector<uint32_t> deg(V + 1, 0), adj(3 * (size_t)F);
  for (size_t i = 0; i < 3 * (size_t)F; ++i) deg[fv[i] + 1]++;
  for (uint32_t v = 0; v < V; ++v) deg[v + 1] += deg[v];
  {
    std::vector<uint32_t> fill(deg.begin(), deg.end() - 1);
    for (uint32_t f = 0; f < F; ++f)
      for (int j = 0; j < 3; ++j) adj[fill[fv[3 * (size_t)f + j]]++] = f;
  }
  std::vector<uint8_t> assigned(F, 0);
  std::vector<uint32_t> stamp(V, 0xffffffffu), local(V, 0);
  std::vector<uint32_t> queue;
  uint32_t mid = 0;
  for (uint32_t seed = 0; seed < F; ++seed) {
    if (assigned[seed]) continue;
    std::vector<uint32_t> verts, faces;
    queue.clear();
    queue.push_back(seed);
    for (size_t qi = 0; qi < queue.size() && faces.size() < (size_t)cap; ++qi) {
      const uint32_t f = queue[qi];
      if (assigned[f]) continue;
      int fresh = 0;
      for (int j = 0; j < 3; ++j) fresh += stamp[fv[3 * (size_t)f + j]] != mid;
      if (verts.size() + fresh > (size_t)cap) continue;
      assigned[f] = 1;
      faces.push_back(f);
      for (int j = 0; j < 3; ++j) {
        const uint32_t v = fv[3 * (size_t)f + j];
        if (stamp[v] != mid) {
          stamp[v] = mid;
          local[v] = (uint32_t)verts.size();
          verts.push_back(v);
        }
        for (uint32_t a = deg[v]; a < deg[v + 1]; ++a)
          if (!assigned[adj[a]]) queue.push_back(adj[a]);
      }
    }
    MeshletHdr h;
    h.off = (uint32_t)blob.size();
    h.nv = (uint16_t)verts.size();
    h.nf = (uint16_t)faces.size();
    const size_t bytes = verts.size() * 16 + mlet_align16(faces.size() * 4);
    blob.resize(blob.size() + bytes, 0);
    float* pv = reinterpret_cast<float*>(blob.data() + h.off);
    for (size_t i = 0; i < verts.size(); ++i) {
      pv[4 * i + 0] = pos[3 * (size_t)verts[i] + 0];
      pv[4 * i + 1] = pos[3 * (size_t)verts[i] + 1];
      pv[4 * i + 2] = pos[3 * (size_t)verts[i] + 2];
      pv[4 * i + 3] = 0.f;
    }
    uint32_t* pf = reinterpret_cast<uint32_t*>(blob.data() + h.off + verts.size() * 16);
    for (size_t i = 0; i < faces.size(); ++i) {
      const uint32_t f = faces[i];
      pf[i] = local[fv[3 * (size_t)f]] | (local[fv[3 * (size_t)f + 1]] << 10) |
              (local[fv[3 * (size_t)f + 2]] << 20);
    }
    hdr.push_back(h);
    ++mid;
  }
  *box_off = blob.size();
  const size_t ng = (hdr.size() + kMletGroup - 1) / kMletGroup;
  blob.resize(blob.size() + (hdr.size() + ng) * 32, 0);
  for (size_t i = 0; i < hdr.size(); ++i) {
    const float* pv = reinterpret_cast<const float*>(blob.data() + hdr[i].off);
    float b[8] = {pv[0], pv[1], pv[2], 0.f, pv[0], pv[1], pv[2], 0.f};
    for (uint32_t v = 1; v < hdr[i].nv; ++v)
      for (int c = 0; c < 3; ++c) {
        b[c] = pv[4 * v + c] < b[c] ? pv[4 * v + c] : b[c];
        b[4 + c] = pv[4 * v + c] > b[4 + c] ? pv[4 * v + c] : b[4 + c];
      }
    std::memcpy(blob.data() + *box_off + 32 * i, b, 32);
  }
  // group boxes: the union of each run of kMletGroup consecutive meshlets'
  // boxes (consecutive meshlets are neighbouring surface patches)
  for (size_t g = 0; g < ng; ++g) {
    float u[8];
    std::memcpy(u, blob.data() + *box_off + 32 * (g * kMletGroup), 32);
    for (size_t i = g * kMletGroup + 1; i < std::min(hdr.size(), (g + 1) * (size_t)kMletGroup); ++i) {
      float b[8];
      std::memcpy(b, blob.data() + *box_off + 32 * i, 32);
      for (int c = 0; c < 3; ++c) {
        u[c] = b[c] < u[c] ? b[c] : u[c];
        u[4 + c] = b[4 + c] > u[4 + c] ? b[4 + c] : u[4 + c];
      }
    }
    std::memcpy(blob.data() + *box_off + 32 * (hdr.size() + g), u, 32);
  }
}

}  // namespace qpso
