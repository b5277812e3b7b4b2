// MDS .smb mesh files (one part) and the flattened layout of sprg_mesh_view
// (mds/mds_smb.c:547-637, the pcu encoding of pcu/pcu_io.c:242-336).
//
// Layout, all big-endian (uint32 "unsigned", IEEE float64 "double"):
//   header     magic, version (<= 6), dim, number of parts
//   counts     8 unsigned in SMB type order: vertex, edge, triangle, quad,
//              hex, prism, pyramid, tet
//   connectivity, for each type after the vertex in SMB order: the
//              downward adjacency one dimension down (edge: 2 vertices,
//              triangle: 3 edges, quad: 4 edges, hex: 6 quads, prism: 2
//              triangles + 3 quads, pyramid: 1 quad + 4 triangles, tet: 4
//              triangles), as indices of that type
//   coordinates 3 doubles per vertex
//   then parametric coordinates (version >= 2), remote copies,
//   classification, tags, periodic matches (version >= 3), the apf meta
//   section (version >= 5).
//
// Reader: the header, counts, connectivity and coordinates; the rest does
// not enter the estimate-and-mark pass and is not read.  Only simplex
// meshes are taken: files with quads, hexes, prisms or pyramids are
// refused.  Element vertices follow MDS's derivation from the downward
// adjacency (mds/mds.c:498 common_down, 627-662 convert_down): a tet's
// edges are the common edges of face pairs (0,1) (0,2) (0,3) (1,3) (1,2)
// (2,3), its vertices the common vertices of edge pairs (2,0) (0,1) (1,2)
// (3,4); a triangle's vertices those of its edge pairs (2,0) (0,1) (1,2).
//
// Writer: version 4 (no meta section); the flattened edges, the triangles
// of the elements numbered in order of first appearance (element order,
// faces in the canonical order (0,1,2) (0,1,3) (1,2,3) (0,2,3) of
// apf/apfMesh.cc, their edges (0,1) (1,2) (2,0)), so that the derivation
// above gives back every element's vertex order; every entity classified on
// the model entity of the mesh's dimension with tag 0 (the flattened mesh
// carries no geometric classification); one part, no tags, no matches.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <unordered_map>
#include <utility>
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
  // bytes from the current position to the end of the file, or -1
  int64_t remaining() {
    if (!ok) return -1;
    const long here = std::ftell(f);
    if (here < 0 || std::fseek(f, 0, SEEK_END) != 0) return -1;
    const long end = std::ftell(f);
    if (end < 0 || std::fseek(f, here, SEEK_SET) != 0) return -1;
    return (int64_t)end - here;
  }
};

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
  // the connectivity and coordinates the counts announce must be in the
  // file, so that a short or damaged file sizes no allocation
  const uint64_t need =
      4ull * (2ull * s.n[kEdge] + 3ull * s.n[kTri] + 4ull * s.n[kTet]) + 24ull * s.n[kVert];
  const int64_t have = r.remaining();
  if (have < 0 || (uint64_t)have < need) return SPRG_EINVAL;
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

namespace {

struct Writer {
  FILE* f = nullptr;
  bool ok = true;
  explicit Writer(const char* path) { f = std::fopen(path, "wb"); ok = f != nullptr; }
  ~Writer() {
    if (f) std::fclose(f);
  }
  void u32s(const uint32_t* p, size_t n) {
    if (!ok || !n) return;
    std::vector<unsigned char> b(4 * n);
    for (size_t i = 0; i < n; ++i)
      for (int k = 0; k < 4; ++k) b[4 * i + k] = (unsigned char)(p[i] >> (24 - 8 * k));
    ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
  }
  void u32(uint32_t x) { u32s(&x, 1); }
  void f64s(const double* p, size_t n) {
    if (!ok || !n) return;
    std::vector<unsigned char> b(8 * n);
    for (size_t i = 0; i < n; ++i) {
      uint64_t u;
      std::memcpy(&u, p + i, 8);
      for (int k = 0; k < 8; ++k) b[8 * i + k] = (unsigned char)(u >> (56 - 8 * k));
    }
    ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
  }
};

uint64_t pair_key(uint32_t a, uint32_t b) {
  if (a > b) std::swap(a, b);
  return (uint64_t)a << 32 | b;
}

struct FaceKey {
  uint32_t e[3];
  bool operator==(const FaceKey& o) const { return e[0] == o.e[0] && e[1] == o.e[1] && e[2] == o.e[2]; }
};
struct FaceKeyHash {
  size_t operator()(const FaceKey& k) const {
    uint64_t h = k.e[0];
    h = h * 0x9E3779B97F4A7C15ull ^ k.e[1];
    h = h * 0x9E3779B97F4A7C15ull ^ k.e[2];
    return (size_t)(h ^ (h >> 29));
  }
};

}  // namespace

extern "C" int sprg_smb_write(const char* path, const sprg_mesh_view* mv) {
  if (!path || !mv || (mv->dim != 2 && mv->dim != 3) || mv->n_verts <= 0 || mv->n_elems <= 0 || mv->n_edges <= 0 ||
      !mv->coords || !mv->elem_verts || !mv->edge_verts)
    return SPRG_EINVAL;
  if (mv->n_verts >= kMaxEntities || mv->n_edges >= kMaxEntities || mv->n_elems >= kMaxEntities) return SPRG_EINVAL;
  const uint32_t V = (uint32_t)mv->n_verts, E = (uint32_t)mv->n_edges, T = (uint32_t)mv->n_elems;
  const int nn = mv->dim + 1;
  std::unordered_map<uint64_t, uint32_t> edge_of;
  edge_of.reserve(2 * (size_t)E);
  std::vector<uint32_t> edges(2 * (size_t)E);
  for (uint32_t e = 0; e < E; ++e) {
    const int32_t a = mv->edge_verts[2 * (size_t)e], b = mv->edge_verts[2 * (size_t)e + 1];
    if (a < 0 || b < 0 || (uint32_t)a >= V || (uint32_t)b >= V || a == b) return SPRG_EINVAL;
    edges[2 * (size_t)e] = (uint32_t)a;
    edges[2 * (size_t)e + 1] = (uint32_t)b;
    if (!edge_of.emplace(pair_key(a, b), e).second) return SPRG_EINVAL;  // duplicate edge
  }
  static const int tri_edge[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  static const int tet_tri[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
  // triangles: the elements themselves (2D) or the tets' faces (3D)
  std::vector<uint32_t> tris, tet_faces;
  auto tri_edges = [&](const uint32_t* v, uint32_t* out) {
    for (int i = 0; i < 3; ++i) {
      auto it = edge_of.find(pair_key(v[tri_edge[i][0]], v[tri_edge[i][1]]));
      if (it == edge_of.end()) return false;
      out[i] = it->second;
    }
    return true;
  };
  if (mv->dim == 2) {
    tris.resize(3 * (size_t)T);
    for (uint32_t t = 0; t < T; ++t) {
      uint32_t v[3];
      for (int i = 0; i < 3; ++i) {
        const int32_t x = mv->elem_verts[3 * (size_t)t + i];
        if (x < 0 || (uint32_t)x >= V) return SPRG_EINVAL;
        v[i] = (uint32_t)x;
      }
      if (!tri_edges(v, &tris[3 * (size_t)t])) return SPRG_EINVAL;
    }
  } else {
    std::unordered_map<FaceKey, uint32_t, FaceKeyHash> face_of;  // the face's three edge ids, sorted
    face_of.reserve(2 * (size_t)T);
    tet_faces.resize(4 * (size_t)T);
    for (uint32_t t = 0; t < T; ++t) {
      uint32_t v[4];
      for (int i = 0; i < 4; ++i) {
        const int32_t x = mv->elem_verts[4 * (size_t)t + i];
        if (x < 0 || (uint32_t)x >= V) return SPRG_EINVAL;
        v[i] = (uint32_t)x;
      }
      for (int f = 0; f < 4; ++f) {
        const uint32_t fv[3] = {v[tet_tri[f][0]], v[tet_tri[f][1]], v[tet_tri[f][2]]};
        uint32_t fe[3];
        if (!tri_edges(fv, fe)) return SPRG_EINVAL;
        FaceKey k{{fe[0], fe[1], fe[2]}};
        if (k.e[0] > k.e[1]) std::swap(k.e[0], k.e[1]);
        if (k.e[1] > k.e[2]) std::swap(k.e[1], k.e[2]);
        if (k.e[0] > k.e[1]) std::swap(k.e[0], k.e[1]);
        auto ins = face_of.emplace(k, (uint32_t)(tris.size() / 3));
        if (ins.second) tris.insert(tris.end(), fe, fe + 3);
        const uint32_t id = ins.first->second;
        tet_faces[4 * (size_t)t + f] = id;
      }
    }
  }
  const uint32_t F = (uint32_t)(tris.size() / 3);
  const uint32_t Tt = mv->dim == 3 ? T : 0;
  Writer w(path);
  const uint32_t counts[kTypes] = {V, E, F, 0, 0, 0, 0, Tt};
  w.u32(0);  // magic
  w.u32(4);  // version
  w.u32((uint32_t)mv->dim);
  w.u32(1);  // one part
  w.u32s(counts, kTypes);
  w.u32s(edges.data(), edges.size());
  w.u32s(tris.data(), tris.size());
  w.u32s(tet_faces.data(), tet_faces.size());
  w.f64s(mv->coords, 3 * (size_t)V);
  std::vector<double> params(2 * (size_t)V, 0.0);
  w.f64s(params.data(), params.size());
  w.u32(0);  // remote copies: no peers
  for (int t = 0; t < kTypes; ++t) {  // classification: (tag 0, dimension of the mesh)
    std::vector<uint32_t> cls(2 * (size_t)counts[t]);
    for (size_t j = 0; j < counts[t]; ++j) cls[2 * j + 1] = (uint32_t)mv->dim;
    w.u32s(cls.data(), cls.size());
  }
  w.u32(0);                                       // no tags (no per-type tag sizes follow)
  for (int t = 0; t < kTypes; ++t) w.u32(0);      // periodic matches: no peers
  return w.ok ? SPRG_OK : SPRG_EINVAL;
}
