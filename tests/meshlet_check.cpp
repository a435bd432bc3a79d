// Checks the meshlet partition (q-pso_gb300/csrc/meshlets.h) of a mesh read
// from a binary file of 9*F floats (loadOBJ3 layout): every face exactly
// once, caps respected, local ids inside the meshlet, positions preserved,
// each meshlet's box the exact bounds of its vertices, each group box the
// union of its meshlets' boxes.
// Prints "faces meshlets unique_vertex_slots cap".
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "meshlets.h"

int main(int argc, char** argv) {
  if (argc != 2) return 2;
  FILE* fp = std::fopen(argv[1], "rb");
  if (!fp) return 2;
  std::vector<float> soa;
  float buf[4096];
  size_t n;
  while ((n = std::fread(buf, 4, 4096, fp)) > 0) soa.insert(soa.end(), buf, buf + n);
  std::fclose(fp);
  const uint32_t F = (uint32_t)(soa.size() / 9);
  std::vector<qpso::MeshletHdr> hdr;
  std::vector<unsigned char> blob;
  size_t box_off = 0;
  const int cap = qpso::meshlet_cap(F);
  qpso::build_meshlets(soa.data(), F, hdr, blob, &box_off, cap);
  const size_t ng = (hdr.size() + qpso::kMletGroup - 1) / qpso::kMletGroup;
  if (box_off % 16 != 0 || blob.size() != box_off + 32 * (hdr.size() + ng)) return 7;
  // every group box is the union of its meshlets' boxes
  const float* boxes = reinterpret_cast<const float*>(blob.data() + box_off);
  for (size_t g = 0; g < ng; ++g) {
    float u[6] = {3e38f, 3e38f, 3e38f, -3e38f, -3e38f, -3e38f};
    for (size_t i = g * qpso::kMletGroup; i < hdr.size() && i < (g + 1) * qpso::kMletGroup; ++i)
      for (int c = 0; c < 3; ++c) {
        u[c] = std::min(u[c], boxes[8 * i + c]);
        u[3 + c] = std::max(u[3 + c], boxes[8 * i + 4 + c]);
      }
    const float* gb = boxes + 8 * (hdr.size() + g);
    for (int c = 0; c < 3; ++c)
      if (gb[c] != u[c] || gb[4 + c] != u[3 + c]) return 9;
  }
  // multiset of faces as (x,y,z) x 3 -> compare counts by summing a hash
  uint64_t want = 0, got = 0, slots = 0, faces = 0;
  auto fh = [](const float* a, const float* b, const float* c) {
    uint64_t h = 1469598103934665603ull;
    const float* v[3] = {a, b, c};
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) {
        uint32_t u;
        std::memcpy(&u, &v[j][k], 4);
        h = (h ^ u) * 1099511628211ull;
      }
    return h;
  };
  for (uint32_t f = 0; f < F; ++f) {
    float a[3], b[3], c[3];
    for (int k = 0; k < 3; ++k) {
      a[k] = soa[f + (size_t)(3 * k + 0) * F];
      b[k] = soa[f + (size_t)(3 * k + 1) * F];
      c[k] = soa[f + (size_t)(3 * k + 2) * F];
    }
    want += fh(a, b, c);
  }
  for (const auto& h : hdr) {
    if (h.nv == 0 || h.nf == 0 || h.nv > cap || h.nf > cap) return 3;
    if (h.off % 16 != 0) return 4;
    const float* pv = reinterpret_cast<const float*>(blob.data() + h.off);
    const uint32_t* pf = reinterpret_cast<const uint32_t*>(blob.data() + h.off + h.nv * 16);
    for (int i = 0; i < h.nf; ++i) {
      const uint32_t a = pf[i] & 1023u, b = (pf[i] >> 10) & 1023u, c = (pf[i] >> 20) & 1023u;
      if (a >= h.nv || b >= h.nv || c >= h.nv) return 5;
      got += fh(pv + 4 * a, pv + 4 * b, pv + 4 * c);
    }
    const float* bx = reinterpret_cast<const float*>(blob.data() + box_off) + 8 * (&h - hdr.data());
    for (int c = 0; c < 3; ++c) {
      bool lo_hit = false, hi_hit = false;
      for (int v = 0; v < h.nv; ++v) {
        if (pv[4 * v + c] < bx[c] || pv[4 * v + c] > bx[4 + c]) return 8;
        lo_hit |= pv[4 * v + c] == bx[c];
        hi_hit |= pv[4 * v + c] == bx[4 + c];
      }
      if (!lo_hit || !hi_hit) return 8;
    }
    slots += h.nv;
    faces += h.nf;
  }
  if (faces != F || got != want) return 6;
  std::printf("%u %zu %llu %d\n", F, hdr.size(), (unsigned long long)slots, cap);
  return 0;
}
