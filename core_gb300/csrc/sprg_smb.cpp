// One part of an MDS .smb mesh file read straight into the flattened layout
// of sprg_mesh_view (mds/mds_smb.c:547-606, the pcu encoding of
// pcu/pcu_io.c:242-336).
//
// Layout of the parts read here, all big-endian (uint32 "unsigned",
// IEEE float64 "double"):
//   header     magic, version (<= 6), dim, number of parts
//   counts     8 unsigned in SMB type order: vertex, edge, triangle, quad,
//              hex, prism, pyramid, tet
//   connectivity, for each type after the vertex in SMB order: the
//              downward adjacency one dimension down (edge: 2 vertices,
//              triangle: 3 edges, quad: 4 edges, hex: 6 quads, prism: 2
//              triangles + 3 quads, pyramid: 1 quad + 4 triangles, tet: 4
//              triangles), as indices of that type
//   coordinates 3 doubles per vertex
// What follows (parametric coordinates from version 2, remote copies,
// classification, tags, periodic matches, the apf meta section from
// version 5) does not enter the estimate-and-mark pass and is not read.
//
// Only simplex meshes are taken: files with quads, hexes, prisms or
// pyramids are refused.  Element vertices follow MDS's derivation from the
// downward adjacency (mds/mds.c:498 common_down, 627-662 convert_down): a
// tet's edges are the common edges of face pairs (0,1) (0,2) (0,3) (1,3)
// (1,2) (2,3), its vertices the common vertices of edge pairs (2,0) (0,1)
// (1,2) (3,4); a triangle's vertices those of its edge pairs (2,0) (0,1)
// (1,2).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "spr_gb300.h"

namespace {

enum { kVert, kEdge, kTri, kQuad, kHex, kPrism, kPyr, kTet, kTypes };
constexpr uint32_t kMaxVersion = 6;
constexpr uint32_t kMaxEntities = 100u * 1000u * 1000u;

struct Reader {
  FILE* f = nullptr;
  bool ok = true;
  explicit Reader(const char* path) { f = std::fopen(path, "rb"); ok = f != nullptr; }
  ~Reader() {
    if (f) std::fclose(f);
  }
  bool u32s(uint32_t* p, size_t n) {
    if (!ok) return false;
    std::vector<unsigned char> b(4 * n);
    if (n && std::fread(b.data(), 1, b.size(), f) != b.size()) return ok = false;
    for (size_t i = 0; i < n; ++i)
      p[i] = (uint32_t)b[4 * i] << 24 | (uint32_t)b[4 * i + 1] << 16 | (uint32_t)b[4 * i + 2] << 8 |
             (uint32_t)b[4 * i + 3];
    return true;
  }
  bool f64s(double* p, size_t n) {
    if (!ok) return false;
    std::vector<unsigned char> b(8 * n);
    if (n && std::fread(b.data(), 1, b.size(), f) != b.size()) return ok = false;
    for (size_t i = 0; i < n; ++i) {
      uint64_t u = 0;
      for (int k = 0; k < 8; ++k) u = u << 8 | b[8 * i + k];
      std::memcpy(p + i, &u, 8);
    }
    return true;
  }
};

// downward degree of each SMB type (one dimension down)
constexpr int kDownDegree[kTypes] = {0, 2, 3, 4, 6, 5, 5, 4};

struct SmbMesh {
  uint32_t version = 0, dim = 0;
  uint32_t n[kTypes] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<uint32_t> edge_verts, tri_edges, tet_tris;
  std::vector<double> coords;
};

int read_smb(const char* path, SmbMesh& s, bool with_arrays) {
  if (!path) return SPRG_EINVAL;
  Reader r(path);
  if (!r.ok) return SPRG_EINVAL;
  uint32_t head[4];
  if (!r.u32s(head, 4)) return SPRG_EINVAL;
  s.version = head[1];
  s.dim = head[2];
  if (s.version > kMaxVersion || (s.dim != 2 && s.dim != 3)) return SPRG_EINVAL;
  if (!r.u32s(s.n, kTypes)) return SPRG_EINVAL;
  for (int t = 0; t < kTypes; ++t)
    if (s.n[t] >= kMaxEntities) return SPRG_EINVAL;
  if (s.n[kQuad] || s.n[kHex] || s.n[kPrism] || s.n[kPyr]) return SPRG_EINVAL;  // simplex meshes only
  if ((s.dim == 3 && (!s.n[kTet] || !s.n[kTri])) || (s.dim == 2 && (s.n[kTet] || !s.n[kTri])) || !s.n[kEdge] ||
      !s.n[kVert])
    return SPRG_EINVAL;
  if (!with_arrays) return SPRG_OK;
  try {
    s.edge_verts.resize(2 * (size_t)s.n[kEdge]);
    s.tri_edges.resize(3 * (size_t)s.n[kTri]);
    s.tet_tris.resize(4 * (size_t)s.n[kTet]);
    s.coords.resize(3 * (size_t)s.n[kVert]);
  } catch (...) {
    return SPRG_ENOMEM;
  }
  // connectivity in SMB type order; the refused types have no rows
  if (!r.u32s(s.edge_verts.data(), s.edge_verts.size()) || !r.u32s(s.tri_edges.data(), s.tri_edges.size()) ||
      !r.u32s(s.tet_tris.data(), s.tet_tris.size()) || !r.f64s(s.coords.data(), s.coords.size()))
    return SPRG_EINVAL;
  for (uint32_t v : s.edge_verts)
    if (v >= s.n[kVert]) return SPRG_EINVAL;
  for (uint32_t e : s.tri_edges)
    if (e >= s.n[kEdge]) return SPRG_EINVAL;
  for (uint32_t t : s.tet_tris)
    if (t >= s.n[kTri]) return SPRG_EINVAL;
  return SPRG_OK;
}

// the single entity both downward lists share (mds common_down)
bool common(const uint32_t* a, const uint32_t* b, int n, uint32_t* out) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      if (a[i] == b[j]) {
        *out = a[i];
        return true;
      }
  return false;
}

}  // namespace

extern "C" int sprg_smb_counts(const char* path, int* dim, int64_t* n_verts, int64_t* n_elems, int64_t* n_edges) {
  if (!dim || !n_verts || !n_elems || !n_edges) return SPRG_EINVAL;
  SmbMesh s;
  const int rc = read_smb(path, s, false);
  if (rc) return rc;
  *dim = (int)s.dim;
  *n_verts = s.n[kVert];
  *n_elems = s.dim == 3 ? s.n[kTet] : s.n[kTri];
  *n_edges = s.n[kEdge];
  return SPRG_OK;
}

extern "C" int sprg_smb_read(const char* path, double* coords, int32_t* elem_verts, int32_t* edge_verts) {
  if (!coords || !elem_verts || !edge_verts) return SPRG_EINVAL;
  SmbMesh s;
  const int rc = read_smb(path, s, true);
  if (rc) return rc;
  std::memcpy(coords, s.coords.data(), sizeof(double) * s.coords.size());
  for (size_t i = 0; i < s.edge_verts.size(); ++i) edge_verts[i] = (int32_t)s.edge_verts[i];
  static const int t10[3][2] = {{2, 0}, {0, 1}, {1, 2}};
  if (s.dim == 2) {
    for (uint32_t t = 0; t < s.n[kTri]; ++t) {
      const uint32_t* e = &s.tri_edges[3 * (size_t)t];
      for (int i = 0; i < 3; ++i) {
        uint32_t v;
        if (!common(&s.edge_verts[2 * (size_t)e[t10[i][0]]], &s.edge_verts[2 * (size_t)e[t10[i][1]]], 2, &v))
          return SPRG_EINVAL;
        elem_verts[3 * (size_t)t + i] = (int32_t)v;
      }
    }
    return SPRG_OK;
  }
  static const int T21[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 3}, {1, 2}, {2, 3}};
  static const int T10[4][2] = {{2, 0}, {0, 1}, {1, 2}, {3, 4}};
  for (uint32_t t = 0; t < s.n[kTet]; ++t) {
    const uint32_t* f = &s.tet_tris[4 * (size_t)t];
    uint32_t ed[6];
    for (int i = 0; i < 6; ++i)
      if (!common(&s.tri_edges[3 * (size_t)f[T21[i][0]]], &s.tri_edges[3 * (size_t)f[T21[i][1]]], 3, &ed[i]))
        return SPRG_EINVAL;
    for (int i = 0; i < 4; ++i) {
      uint32_t v;
      if (!common(&s.edge_verts[2 * (size_t)ed[T10[i][0]]], &s.edge_verts[2 * (size_t)ed[T10[i][1]]], 2, &v))
        return SPRG_EINVAL;
      elem_verts[4 * (size_t)t + i] = (int32_t)v;
    }
  }
  return SPRG_OK;
}
