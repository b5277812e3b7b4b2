// Flattened apf::makeMdsBox (mds/apfBox.cc:68-330).
//
// BoxBuilder creates vertices in grid order, then the grid edges of every
// vertex (+x, +y, +z), then two triangles per quad face, whose first
// triangle (v0,v1,v2) creates the face diagonal as the edge (v2,v0), then
// six tets per cube around the diagonal 0-6, whose second face (0,1,6)
// creates that diagonal as the edge (6,0).  MDS numbers entities of a
// dimension in creation order (mds/mds.c:520 alloc_ent), so every index
// and every stored vertex order below follows from the loop order alone;
// no hashing or find-or-create is needed.
#include <cstdint>

#include "spr_gb300.h"

namespace {

struct Grid {
  int n[3];
  long s[3];  // grid sizes n+1
  long idx(long x, long y, long z) const { return x + s[0] * (y + s[1] * z); }
};

}  // namespace

extern "C" int sprg_box_counts(int nx, int ny, int nz, int64_t* n_verts, int64_t* n_elems, int64_t* n_edges) {
  if (nx < 1 || ny < 1 || nz < 0 || !n_verts || !n_elems || !n_edges) return SPRG_EINVAL;
  int64_t X = nx, Y = ny, Z = nz;
  if (nz == 0) {
    *n_verts = (X + 1) * (Y + 1);
    *n_elems = 2 * X * Y;
    *n_edges = X * (Y + 1) + (X + 1) * Y + X * Y;
  } else {
    *n_verts = (X + 1) * (Y + 1) * (Z + 1);
    *n_elems = 6 * X * Y * Z;
    *n_edges = X * (Y + 1) * (Z + 1) + (X + 1) * Y * (Z + 1) + (X + 1) * (Y + 1) * Z  // grid edges
               + X * Y * (Z + 1) + Y * Z * (X + 1) + Z * X * (Y + 1)                   // face diagonals
               + X * Y * Z;                                                             // cube diagonals
  }
  return SPRG_OK;
}

extern "C" int sprg_box_fill(int nx, int ny, int nz, double wx, double wy, double wz, double* coords,
                             int32_t* elem_verts, int32_t* edge_verts) {
  int64_t V, T, E;
  int rc = sprg_box_counts(nx, ny, nz, &V, &T, &E);
  if (rc) return rc;
  if (!coords || !elem_verts || !edge_verts) return SPRG_EINVAL;
  if (V > INT32_MAX || E > INT32_MAX || T > INT32_MAX) return SPRG_EINVAL;
  Grid g{{nx, ny, nz}, {nx + 1L, ny + 1L, nz + 1L}};
  const int dim = nz ? 3 : 2;
  const double w[3] = {wx / nx, wy / ny, nz ? (wz / nz) : 0};
  // vertices (BoxBuilder::buildCellVert)
  for (long z = 0; z < g.s[2]; ++z)
    for (long y = 0; y < g.s[1]; ++y)
      for (long x = 0; x < g.s[0]; ++x) {
        long v = g.idx(x, y, z);
        coords[3 * v + 0] = w[0] * (int)x;
        coords[3 * v + 1] = w[1] * (int)y;
        coords[3 * v + 2] = w[2] * (int)z;
      }
  long e = 0;
  // grid edges (BoxBuilder::buildCellEdges)
  for (long z = 0; z < g.s[2]; ++z)
    for (long y = 0; y < g.s[1]; ++y)
      for (long x = 0; x < g.s[0]; ++x) {
        long v = g.idx(x, y, z);
        long c[3] = {x, y, z};
        for (int j = 0; j < 3; ++j) {
          if (c[j] >= g.n[j]) continue;  // model index 2 (or the flat z of a 2D box)
          long o[3] = {x, y, z};
          o[j] += 1;
          edge_verts[2 * e] = (int32_t)v;
          edge_verts[2 * e + 1] = (int32_t)g.idx(o[0], o[1], o[2]);
          ++e;
        }
      }
  // quad faces -> 2 triangles; the first creates the diagonal (v2, v0)
  long t = 0;
  for (long z = 0; z < g.s[2]; ++z)
    for (long y = 0; y < g.s[1]; ++y)
      for (long x = 0; x < g.s[0]; ++x) {
        long c[3] = {x, y, z};
        for (int jx = 0; jx < 3; ++jx) {
          int jy = (jx + 1) % 3;
          if (c[jx] >= g.n[jx] || c[jy] >= g.n[jy]) continue;
          long b[3] = {x, y, z}, cc[3], d[3] = {x, y, z};
          b[jx] += 1;
          cc[0] = b[0]; cc[1] = b[1]; cc[2] = b[2];
          cc[jy] += 1;
          d[jy] += 1;
          long f0 = g.idx(x, y, z), f1 = g.idx(b[0], b[1], b[2]), f2 = g.idx(cc[0], cc[1], cc[2]),
               f3 = g.idx(d[0], d[1], d[2]);
          edge_verts[2 * e] = (int32_t)f2;
          edge_verts[2 * e + 1] = (int32_t)f0;
          ++e;
          if (dim == 2) {
            int32_t* tv = elem_verts + 3 * t;
            tv[0] = (int32_t)f0; tv[1] = (int32_t)f1; tv[2] = (int32_t)f2;
            tv[3] = (int32_t)f2; tv[4] = (int32_t)f3; tv[5] = (int32_t)f0;
            t += 2;
          }
        }
      }
  if (dim == 3) {
    static const int tv6[6][4] = {{0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}, {0, 5, 1, 6}};
    for (long z = 0; z < g.n[2]; ++z)
      for (long y = 0; y < g.n[1]; ++y)
        for (long x = 0; x < g.n[0]; ++x) {
          long rv[8] = {g.idx(x, y, z),         g.idx(x + 1, y, z),     g.idx(x + 1, y + 1, z),
                        g.idx(x, y + 1, z),     g.idx(x, y, z + 1),     g.idx(x + 1, y, z + 1),
                        g.idx(x + 1, y + 1, z + 1), g.idx(x, y + 1, z + 1)};
          edge_verts[2 * e] = (int32_t)rv[6];
          edge_verts[2 * e + 1] = (int32_t)rv[0];
          ++e;
          for (int k = 0; k < 6; ++k)
            for (int j = 0; j < 4; ++j) elem_verts[4 * (t + k) + j] = (int32_t)rv[tv6[k][j]];
          t += 6;
        }
  }
  return (e == E && t == T) ? SPRG_OK : SPRG_EINVAL;
}
