/*
 * spr_oracle.c -- CPU restatement of PUMI's estimate-and-mark path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path in
 * core_gb300/: it is imported by tests/, by __graft_entry__.smoke() and by
 * bench.py's cpu_baseline / --impl reference legs, and by nothing else.  It
 * is never linked into, called by, or shipped with the product library.
 *
 * It restates, in plain C99 FP64 with FMA contraction disabled
 * (-ffp-contract=off), the algorithms of SCOREC/core (reference tree paths
 * below are relative to that project's root):
 *
 *   mesh numbering / adjacency   mds/mds.c, apf/apfMesh.cc, apf/apfMesh2.cc
 *   box generator                mds/apfBox.cc
 *   gradient at int. points      spr/sprGetGradIPField.cc
 *   SPR patch recovery           spr/sprRecoverField.cc, mth/mthQR.cc
 *   SPR size field               spr/sprEstimateError.cc
 *   target SPR size field        spr/sprEstimateTargetError.cc
 *   metric edge length           ma/maSize.cc
 *   edge marking                 ma/maAdapt.cc, ma/maRefine.cc, ma/maCoarsen.cc
 *   mean-ratio quality           ma/maQuality.cc
 *
 * Floating-point operations follow the reference's evaluation order (the
 * operator bodies in apf/apfVector.h, apf/apfMatrix.h, apf/apfMatrix.cc,
 * apf/apfElement.cc, mth/mthQR.cc) so that, compiled without FMA
 * contraction, results are bitwise those of the reference on the same
 * platform libm.
 *
 * Parity pinning: the reference's estimate-and-mark path is compiled from
 * its sources (oracle/Makefile refall -> oracle/_ref/libspr_ref.so) and this
 * restatement equals it bitwise on box numbering, IP gradients, recovered
 * and size fields, edge lengths, qualities and ma_flags words
 * (tests/test_reference_pin.py, and tests/golden/ref_path.npz for hosts
 * without the reference tree); the QR/rank kernel (orc_qr_*) is also pinned
 * against the reference's known-answer test (test/qr.cc) and against
 * mth/mthQR.cc compiled alone (oracle/Makefile ref).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_EPATCH 2
#define ORC_EFLAGS 3
#define ORC_ENOMEM 4
#define ORC_EEIGEN 5

/* ------------------------------------------------------------------ */
/* small vector / matrix helpers, in the reference's evaluation order  */
/* ------------------------------------------------------------------ */

typedef struct { double v[3]; } V3;
typedef struct { double m[3][3]; } M3;

/* apf::Vector<N>::operator* (dot): r=0; r += a[i]*b[i]  (apf/apfVector.h:103) */
static double v3_dot(V3 a, V3 b) {
  double r = 0;
  for (int i = 0; i < 3; ++i) r += a.v[i] * b.v[i];
  return r;
}
static double v3_len(V3 a) { return sqrt(v3_dot(a, a)); }
static V3 v3_scale(V3 a, double s) { V3 c; for (int i = 0; i < 3; ++i) c.v[i] = a.v[i] * s; return c; }
static V3 v3_div(V3 a, double s) { V3 c; for (int i = 0; i < 3; ++i) c.v[i] = a.v[i] / s; return c; }
static V3 v3_add(V3 a, V3 b) { V3 c; for (int i = 0; i < 3; ++i) c.v[i] = a.v[i] + b.v[i]; return c; }
static V3 v3_sub(V3 a, V3 b) { V3 c; for (int i = 0; i < 3; ++i) c.v[i] = a.v[i] - b.v[i]; return c; }
/* apf::cross (apf/apfVector.h:123) */
static V3 v3_cross(V3 a, V3 b) {
  V3 r;
  r.v[0] = a.v[1] * b.v[2] - a.v[2] * b.v[1];
  r.v[1] = a.v[2] * b.v[0] - a.v[0] * b.v[2];
  r.v[2] = a.v[0] * b.v[1] - a.v[1] * b.v[0];
  return r;
}
static V3 v3_normalize(V3 a) { return v3_div(a, v3_len(a)); }

static M3 m3_transpose(M3 a) {
  M3 r;
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[j][i] = a.m[i][j];
  return r;
}
/* apf::Matrix::operator*(Matrix) (apf/apfMatrix.h:95) */
static M3 m3_mul(M3 a, M3 b) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      r.m[i][j] = a.m[i][0] * b.m[0][j];
      for (int k = 1; k < 3; ++k) r.m[i][j] += a.m[i][k] * b.m[k][j];
    }
  return r;
}
/* apf::Matrix::operator*(Vector): row dot products (apf/apfMatrix.h:83) */
static V3 m3_mulv(M3 a, V3 b) {
  V3 r;
  for (int i = 0; i < 3; ++i) {
    V3 row = {{a.m[i][0], a.m[i][1], a.m[i][2]}};
    r.v[i] = v3_dot(row, b);
  }
  return r;
}
static V3 m3_row(M3 a, int i) { V3 r = {{a.m[i][0], a.m[i][1], a.m[i][2]}}; return r; }
static void m3_setrow(M3* a, int i, V3 r) { for (int j = 0; j < 3; ++j) a->m[i][j] = r.v[j]; }

/* apf::getDeterminant, cofactor expansion down column 0 (apf/apfMatrix.cc:85-125) */
static double det2(double a00, double a01, double a10, double a11) {
  double d = 0;
  d += a00 * (1 * a11);
  d += a10 * (-1 * a01);
  return d;
}
static double m3_det(M3 a) {
  double d = 0;
  d += a.m[0][0] * (1 * det2(a.m[1][1], a.m[1][2], a.m[2][1], a.m[2][2]));
  d += a.m[1][0] * (-1 * det2(a.m[0][1], a.m[0][2], a.m[2][1], a.m[2][2]));
  d += a.m[2][0] * (1 * det2(a.m[0][1], a.m[0][2], a.m[1][1], a.m[1][2]));
  return d;
}
/* apf::invert 3x3 (apf/apfMatrix.h:165) */
static M3 m3_invert(M3 m) {
  M3 x = m3_transpose(m), r;
  m3_setrow(&r, 0, v3_cross(m3_row(x, 1), m3_row(x, 2)));
  m3_setrow(&r, 1, v3_cross(m3_row(x, 2), m3_row(x, 0)));
  m3_setrow(&r, 2, v3_cross(m3_row(x, 0), m3_row(x, 1)));
  double d = m3_det(m);
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = r.m[i][j] / d;
  return r;
}
/* apf::getJacobianInverse (apf/apfElement.cc:43-76), dims 2 and 3 */
static M3 jacobian_inverse(M3 J, int dim) {
  if (dim == 3) return m3_invert(J);
  /* dim 2: Moore-Penrose pseudo inverse  transpose(At * invert(A*At)) */
  double A[2][3], At[3][2], AAt[2][2], inv[2][2], AtInv[3][2];
  for (int j = 0; j < 3; ++j) { A[0][j] = J.m[0][j]; A[1][j] = J.m[1][j]; }
  for (int i = 0; i < 2; ++i) for (int j = 0; j < 3; ++j) At[j][i] = A[i][j];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      AAt[i][j] = A[i][0] * At[0][j];
      for (int k = 1; k < 3; ++k) AAt[i][j] += A[i][k] * At[k][j];
    }
  /* apf::invert 2x2 (apf/apfMatrix.h:156) */
  double d = det2(AAt[0][0], AAt[0][1], AAt[1][0], AAt[1][1]);
  inv[0][0] = AAt[1][1] / d; inv[0][1] = -AAt[0][1] / d;
  inv[1][0] = -AAt[1][0] / d; inv[1][1] = AAt[0][0] / d;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 2; ++j) {
      AtInv[i][j] = At[i][0] * inv[0][j];
      AtInv[i][j] += At[i][1] * inv[1][j];
    }
  /* Ainvt = transpose(AtInv) (2x3); jinvt rows = Ainvt rows, row 2 zero; jinv = transpose(jinvt) */
  M3 jinv;
  for (int i = 0; i < 3; ++i) {
    jinv.m[i][0] = AtInv[i][0];
    jinv.m[i][1] = AtInv[i][1];
    jinv.m[i][2] = 0;
  }
  return jinv;
}
/* apf::getJacobianDeterminant (apf/apfVectorElement.cc:68) */
static double jacobian_det(M3 J, int dim) {
  if (dim == 3) return m3_det(J);
  if (dim == 2) return v3_len(v3_cross(m3_row(J, 0), m3_row(J, 1)));
  return v3_len(m3_row(J, 0));
}

/* ------------------------------------------------------------------ */
/* MDS-semantics mesh (mds/mds.c)                                      */
/* ------------------------------------------------------------------ */

typedef struct orc_mesh {
  int dim;
  int n[4], cap[4];
  int* dn[4];       /* dn[d][i*(d+1)+j]: j-th downward (dim d-1) entity of entity i of dim d */
  int* up_first[4]; /* up_first[d][i]: newest use of entity i (dim d) by an entity of dim d+1, -1 if none */
  int* up_next[4];  /* up_next[d][use]: next use in the list; use = i*(d+1)+j for entity i of dim d */
  double* xyz;      /* 3 doubles per vertex */
  /* derived, filled by orc_finalize */
  int* elem_verts;  /* n[dim] x (dim+1), MDS getDownward(e,0) order */
  int* elem_edges;  /* n[dim] x (3 or 6), MDS getDownward(e,1) order */
  int* v2e_off;     /* n[0]+1 */
  int* v2e;         /* getAdjacent(v, dim) order (mds get_up union order) */
} orc_mesh;

static int deg_of(int d) { return d + 1; } /* simplices: #down entities of dim d-1 */

static int grow(orc_mesh* m, int d) {
  int nc = m->cap[d] ? m->cap[d] * 2 : 64;
  int deg = deg_of(d);
  if (d > 0) {
    m->dn[d] = (int*)realloc(m->dn[d], sizeof(int) * (size_t)nc * deg);
    m->up_next[d] = (int*)realloc(m->up_next[d], sizeof(int) * (size_t)nc * deg);
    if (!m->dn[d] || !m->up_next[d]) return ORC_ENOMEM;
  } else {
    m->xyz = (double*)realloc(m->xyz, sizeof(double) * 3 * (size_t)nc);
    if (!m->xyz) return ORC_ENOMEM;
  }
  m->up_first[d] = (int*)realloc(m->up_first[d], sizeof(int) * (size_t)nc);
  if (!m->up_first[d]) return ORC_ENOMEM;
  m->cap[d] = nc;
  return ORC_OK;
}

/* mds_create_entity / add_ent / relate_both: new index = count, uses pushed
   at the head of each down entity's up list (mds/mds.c:318-352, 520-577) */
static int create_entity(orc_mesh* m, int d, const int* down) {
  if (m->n[d] == m->cap[d] && grow(m, d)) return -1;
  int i = m->n[d]++;
  m->up_first[d][i] = -1;
  if (d > 0) {
    int deg = deg_of(d);
    for (int j = 0; j < deg; ++j) {
      int use = i * deg + j;
      m->dn[d][use] = down[j];
      m->up_next[d][use] = m->up_first[d - 1][down[j]];
      m->up_first[d - 1][down[j]] = use;
    }
  }
  return i;
}

static int find_in(const int* a, int n, int x) {
  for (int i = 0; i < n; ++i) if (a[i] == x) return i;
  return -1;
}

/* apf::findUpward (apf/apfMesh.cc:528): scan getUp(down[0]) newest first */
static int find_upward(orc_mesh* m, int d, const int* down) {
  int deg = deg_of(d);
  for (int use = m->up_first[d - 1][down[0]]; use != -1; use = m->up_next[d][use]) {
    int u = use / deg;
    const int* d2 = m->dn[d] + (size_t)u * deg;
    int same = 1;
    for (int i = 0; i < deg; ++i) if (find_in(d2, deg, down[i]) < 0) { same = 0; break; }
    if (same) return u;
  }
  return -1;
}

static int make_or_find(orc_mesh* m, int d, const int* down) {
  int e = find_upward(m, d, down);
  if (e >= 0) return e;
  return create_entity(m, d, down);
}

/* canonical tables (apf/apfMesh.cc:27-91, non-Capstone build) */
static const int tri_edge_verts[3][2] = {{0, 1}, {1, 2}, {2, 0}};
static const int tet_tri_verts[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};

/* apf::buildElement -> ElementVertOp::run (apf/apfMesh.cc:547-674, apf/apfMesh2.cc:31-81) */
static int build_element(orc_mesh* m, int d, const int* verts) {
  int down[4];
  if (d == 1) {
    down[0] = verts[0]; down[1] = verts[1];
  } else if (d == 2) {
    for (int i = 0; i < 3; ++i) {
      int ev[2] = {verts[tri_edge_verts[i][0]], verts[tri_edge_verts[i][1]]};
      down[i] = build_element(m, 1, ev);
      if (down[i] < 0) return -1;
    }
  } else {
    for (int i = 0; i < 4; ++i) {
      int fv[3];
      for (int j = 0; j < 3; ++j) fv[j] = verts[tet_tri_verts[i][j]];
      down[i] = build_element(m, 2, fv);
      if (down[i] < 0) return -1;
    }
  }
  return make_or_find(m, d, down);
}

/* mds common_down (mds/mds.c:498) */
static int common_down(const orc_mesh* m, int d, int a, int b) {
  int deg = deg_of(d);
  const int* da = m->dn[d] + (size_t)a * deg;
  const int* db = m->dn[d] + (size_t)b * deg;
  for (int i = 0; i < deg; ++i)
    for (int j = 0; j < deg; ++j)
      if (da[i] == db[j]) return da[i];
  return -1;
}

/* mds convert_down with tables T21/T10 and t10 (mds/mds.c:76-101, 627-662) */
static void elem_down(const orc_mesh* m, int e, int* verts, int* edges) {
  if (m->dim == 3) {
    static const int T21[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 3}, {1, 2}, {2, 3}};
    static const int T10[4][2] = {{2, 0}, {0, 1}, {1, 2}, {3, 4}};
    const int* f = m->dn[3] + (size_t)e * 4;
    for (int i = 0; i < 6; ++i) edges[i] = common_down(m, 2, f[T21[i][0]], f[T21[i][1]]);
    for (int i = 0; i < 4; ++i) verts[i] = common_down(m, 1, edges[T10[i][0]], edges[T10[i][1]]);
  } else {
    static const int t10[3][2] = {{2, 0}, {0, 1}, {1, 2}};
    const int* ed = m->dn[2] + (size_t)e * 3;
    for (int i = 0; i < 3; ++i) edges[i] = ed[i];
    for (int i = 0; i < 3; ++i) verts[i] = common_down(m, 1, edges[t10[i][0]], edges[t10[i][1]]);
  }
}

typedef struct { int n, cap; int* e; } iset;
static void iset_push_unique(iset* s, int x) {
  for (int i = 0; i < s->n; ++i) if (s->e[i] == x) return;
  if (s->n == s->cap) { s->cap = s->cap ? 2 * s->cap : 64; s->e = (int*)realloc(s->e, sizeof(int) * s->cap); }
  s->e[s->n++] = x;
}

/* mds get_up: repeated expand_once with ordered union (mds/mds.c:666-700) */
static void get_up(const orc_mesh* m, int e, int de, int d, iset* out, iset* tmp) {
  out->n = 0;
  iset_push_unique(out, e);
  for (int dim = de; dim < d; ++dim) {
    tmp->n = 0;
    int deg = deg_of(dim + 1);
    for (int i = 0; i < out->n; ++i)
      for (int use = m->up_first[dim][out->e[i]]; use != -1; use = m->up_next[dim + 1][use])
        iset_push_unique(tmp, use / deg);
    iset swap = *out; *out = *tmp; *tmp = swap;
  }
}

void orc_mesh_free(orc_mesh* m) {
  if (!m) return;
  for (int d = 0; d < 4; ++d) { free(m->dn[d]); free(m->up_first[d]); free(m->up_next[d]); }
  free(m->xyz); free(m->elem_verts); free(m->elem_edges); free(m->v2e_off); free(m->v2e);
  free(m);
}

static int finalize(orc_mesh* m) {
  int d = m->dim, T = m->n[d], nv = d + 1, ne = d == 3 ? 6 : 3;
  m->elem_verts = (int*)malloc(sizeof(int) * (size_t)T * nv);
  m->elem_edges = (int*)malloc(sizeof(int) * (size_t)T * ne);
  m->v2e_off = (int*)malloc(sizeof(int) * ((size_t)m->n[0] + 1));
  if (!m->elem_verts || !m->elem_edges || !m->v2e_off) return ORC_ENOMEM;
  for (int e = 0; e < T; ++e) elem_down(m, e, m->elem_verts + (size_t)e * nv, m->elem_edges + (size_t)e * ne);
  iset out = {0, 0, 0}, tmp = {0, 0, 0};
  size_t total = 0, cap = (size_t)T * nv;
  m->v2e = (int*)malloc(sizeof(int) * cap);
  if (!m->v2e) return ORC_ENOMEM;
  for (int v = 0; v < m->n[0]; ++v) {
    m->v2e_off[v] = (int)total;
    get_up(m, v, 0, d, &out, &tmp);
    for (int i = 0; i < out.n; ++i) m->v2e[total++] = out.e[i];
  }
  m->v2e_off[m->n[0]] = (int)total;
  free(out.e); free(tmp.e);
  return ORC_OK;
}

/* apf::makeMdsBox / BoxBuilder (mds/apfBox.cc:68-330), simplex elements */
int orc_box(int nx, int ny, int nz, double wx, double wy, double wz, orc_mesh** out) {
  *out = NULL;
  int gs[3] = {nx + 1, ny + 1, nz + 1};
  int ms[3] = {nx ? 3 : 1, ny ? 3 : 1, nz ? 3 : 1};
  int dim;
  for (dim = 0; dim < 3 && gs[dim] > 1; ++dim);
  if (dim < 2) return ORC_EINVAL;
  double w[3] = {nx ? (wx / nx) : 0, ny ? (wy / ny) : 0, nz ? (wz / nz) : 0};
  long total = (long)gs[0] * gs[1] * gs[2];
  orc_mesh* m = (orc_mesh*)calloc(1, sizeof(orc_mesh));
  if (!m) return ORC_ENOMEM;
  m->dim = dim;
#define GIDX(x, y, z) ((x) + gs[0] * ((y) + gs[1] * (z)))
#define MIDX(i, d) ((i) == 0 ? 0 : ((i) == gs[d] - 1 ? 2 : 1))
  for (long i = 0; i < total; ++i) {
    int vi[3] = {(int)(i % gs[0]), (int)((i / gs[0]) % gs[1]), (int)(i / ((long)gs[0] * gs[1]))};
    int v = create_entity(m, 0, NULL);
    if (v < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
    m->xyz[3 * v + 0] = w[0] * vi[0];
    m->xyz[3 * v + 1] = w[1] * vi[1];
    m->xyz[3 * v + 2] = w[2] * vi[2];
  }
  for (long i = 0; i < total; ++i) {
    int vi[3] = {(int)(i % gs[0]), (int)((i / gs[0]) % gs[1]), (int)(i / ((long)gs[0] * gs[1]))};
    int mi[3] = {MIDX(vi[0], 0), MIDX(vi[1], 1), MIDX(vi[2], 2)};
    for (int j = 0; j < 3; ++j) {
      if (mi[j] == ms[j] - 1) continue;
      int o[3] = {vi[0], vi[1], vi[2]};
      o[j] += 1;
      int ev[2] = {(int)i, GIDX(o[0], o[1], o[2])};
      if (build_element(m, 1, ev) < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
    }
  }
  for (long i = 0; i < total; ++i) {
    int vi[3] = {(int)(i % gs[0]), (int)((i / gs[0]) % gs[1]), (int)(i / ((long)gs[0] * gs[1]))};
    int mi[3] = {MIDX(vi[0], 0), MIDX(vi[1], 1), MIDX(vi[2], 2)};
    for (int jx = 0; jx < 3; ++jx) {
      int jy = (jx + 1) % 3;
      if (mi[jx] == ms[jx] - 1 || mi[jy] == ms[jy] - 1) continue;
      int a[3] = {vi[0], vi[1], vi[2]}, b[3], c[3], dd[3];
      memcpy(b, a, sizeof a); b[jx] += 1;
      memcpy(c, b, sizeof a); c[jy] += 1;
      memcpy(dd, a, sizeof a); dd[jy] += 1;
      int fv[4] = {(int)i, GIDX(b[0], b[1], b[2]), GIDX(c[0], c[1], c[2]), GIDX(dd[0], dd[1], dd[2])};
      int t0[3] = {fv[0], fv[1], fv[2]}, t1[3] = {fv[2], fv[3], fv[0]};
      if (build_element(m, 2, t0) < 0 || build_element(m, 2, t1) < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
    }
  }
  if (dim == 3) {
    static const int tv6[6][4] = {{0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}, {0, 5, 1, 6}};
    for (long i = 0; i < total; ++i) {
      int x = (int)(i % gs[0]), y = (int)((i / gs[0]) % gs[1]), z = (int)(i / ((long)gs[0] * gs[1]));
      if (MIDX(x, 0) == ms[0] - 1 || MIDX(y, 1) == ms[1] - 1 || MIDX(z, 2) == ms[2] - 1) continue;
      int rv[8] = {GIDX(x, y, z), GIDX(x + 1, y, z), GIDX(x + 1, y + 1, z), GIDX(x, y + 1, z),
                   GIDX(x, y, z + 1), GIDX(x + 1, y, z + 1), GIDX(x + 1, y + 1, z + 1), GIDX(x, y + 1, z + 1)};
      for (int t = 0; t < 6; ++t) {
        int tv[4];
        for (int j = 0; j < 4; ++j) tv[j] = rv[tv6[t][j]];
        if (build_element(m, 3, tv) < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
      }
    }
  }
#undef GIDX
#undef MIDX
  if (finalize(m)) { orc_mesh_free(m); return ORC_ENOMEM; }
  *out = m;
  return ORC_OK;
}

/* Mesh from MDS downward arrays in file order (as mds_smb.c reads them:
   entities of each dimension are created in stored order, which fixes both
   their indices and their up-list order).  edges: E x 2 vertex ids,
   faces: F x 3 edge ids, tets (dim 3): T x 4 face ids. */
int orc_from_down(int dim, int nv, const double* xyz, int ne, const int* edges,
                  int nf, const int* faces, int nt, const int* tets, orc_mesh** out) {
  *out = NULL;
  if (dim != 2 && dim != 3) return ORC_EINVAL;
  orc_mesh* m = (orc_mesh*)calloc(1, sizeof(orc_mesh));
  if (!m) return ORC_ENOMEM;
  m->dim = dim;
  for (int v = 0; v < nv; ++v) {
    if (create_entity(m, 0, NULL) < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
    for (int k = 0; k < 3; ++k) m->xyz[3 * v + k] = xyz[3 * v + k];
  }
  for (int e = 0; e < ne; ++e)
    if (create_entity(m, 1, edges + 2 * (size_t)e) < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
  for (int f = 0; f < nf; ++f)
    if (create_entity(m, 2, faces + 3 * (size_t)f) < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
  if (dim == 3)
    for (int t = 0; t < nt; ++t)
      if (create_entity(m, 3, tets + 4 * (size_t)t) < 0) { orc_mesh_free(m); return ORC_ENOMEM; }
  if (finalize(m)) { orc_mesh_free(m); return ORC_ENOMEM; }
  *out = m;
  return ORC_OK;
}

/* accessors */
int orc_dim(const orc_mesh* m) { return m->dim; }
int orc_count(const orc_mesh* m, int d) { return m->n[d]; }
double* orc_coords(orc_mesh* m) { return m->xyz; }
const int* orc_elem_verts(const orc_mesh* m) { return m->elem_verts; }
const int* orc_elem_edges(const orc_mesh* m) { return m->elem_edges; }
const int* orc_edge_verts(const orc_mesh* m) { return m->dn[1]; }
const int* orc_v2e_off(const orc_mesh* m) { return m->v2e_off; }
const int* orc_v2e(const orc_mesh* m) { return m->v2e; }
const int* orc_down(const orc_mesh* m, int d) { return m->dn[d]; }

/* ------------------------------------------------------------------ */
/* element geometry (apf/apfShape.cc Linear, apf/apfVectorElement.cc)   */
/* ------------------------------------------------------------------ */

static V3 vert_xyz(const orc_mesh* m, int v) {
  V3 r = {{m->xyz[3 * v], m->xyz[3 * v + 1], m->xyz[3 * v + 2]}};
  return r;
}

/* linear simplex shape values (apf/apfShape.cc:139-211) */
static void shape_values(int dim, V3 xi, double* N) {
  if (dim == 3) {
    N[0] = 1 - xi.v[0] - xi.v[1] - xi.v[2];
    N[1] = xi.v[0]; N[2] = xi.v[1]; N[3] = xi.v[2];
  } else if (dim == 2) {
    N[0] = 1 - xi.v[0] - xi.v[1];
    N[1] = xi.v[0]; N[2] = xi.v[1];
  } else {
    N[0] = (1.0 - xi.v[0]) / 2.0;
    N[1] = (1.0 + xi.v[0]) / 2.0;
  }
}
static void shape_grads(int dim, V3* g) {
  memset(g, 0, sizeof(V3) * 4);
  if (dim == 3) {
    g[0].v[0] = -1; g[0].v[1] = -1; g[0].v[2] = -1;
    g[1].v[0] = 1; g[2].v[1] = 1; g[3].v[2] = 1;
  } else if (dim == 2) {
    g[0].v[0] = -1; g[0].v[1] = -1;
    g[1].v[0] = 1; g[2].v[1] = 1;
  } else {
    g[0].v[0] = -0.5; g[1].v[0] = 0.5;
  }
}
/* VectorElement::getJacobian -> gradHelper: J = sum_i tensorProduct(gradN_i, x_i)
   (apf/apfVectorElement.cc:44-66) */
static M3 jacobian(const V3* x, int nn, int dim) {
  V3 g[4];
  shape_grads(dim, g);
  M3 J;
  for (int i = 0; i < 3; ++i) m3_setrow(&J, i, v3_scale(x[0], g[0].v[i]));
  for (int n = 1; n < nn; ++n)
    for (int i = 0; i < 3; ++i) m3_setrow(&J, i, v3_add(m3_row(J, i), v3_scale(x[n], g[n].v[i])));
  return J;
}
/* Element::getComponents: c=0; c += node*N (apf/apfElement.cc:93-112) */
static void interp(const double* nodes, int nn, int nc, const double* N, double* c) {
  for (int k = 0; k < nc; ++k) c[k] = 0;
  for (int n = 0; n < nn; ++n)
    for (int k = 0; k < nc; ++k) c[k] += nodes[n * nc + k] * N[n];
}

static V3 ip_point(int dim) {
  /* integration order 1: tet N1 (1/4,1/4,1/4) w 1/6; triangle N1 (1/3,1/3) w 1/2
     (apf/apfIntegrate.cc:135-145, 316-327) */
  V3 p;
  if (dim == 3) { p.v[0] = 0.25; p.v[1] = 0.25; p.v[2] = 0.25; }
  else { p.v[0] = 1. / 3.; p.v[1] = 1. / 3.; p.v[2] = 0; }
  return p;
}
static double ip_weight(int dim) { return dim == 3 ? 1.0 / 6.0 : 1.0 / 2.0; }

static void elem_coords(const orc_mesh* m, int e, V3* x) {
  int nv = m->dim + 1;
  for (int i = 0; i < nv; ++i) x[i] = vert_xyz(m, m->elem_verts[(size_t)e * nv + i]);
}

/* Element::getGlobalGradients (apf/apfElement.cc:77-90) */
static void global_grads(const V3* x, int dim, V3* gg) {
  int nn = dim + 1;
  M3 J = jacobian(x, nn, dim);
  M3 jinv = jacobian_inverse(J, dim);
  V3 lg[4];
  shape_grads(dim, lg);
  for (int i = 0; i < nn; ++i) gg[i] = m3_mulv(jinv, lg[i]);
}

/* ------------------------------------------------------------------ */
/* spr::getGradIPField (spr/sprGetGradIPField.cc:15-65), order 1        */
/*   ncomp_in 1 (SCALAR -> VECTOR ip field) or 3 (VECTOR -> MATRIX)     */
/* ------------------------------------------------------------------ */
int orc_grad_ip(const orc_mesh* m, const double* f, int ncomp_in, double* ip) {
  int dim = m->dim, T = m->n[dim], nn = dim + 1;
  if (ncomp_in != 1 && ncomp_in != 3) return ORC_EINVAL;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < T; ++e) {
    V3 x[4], gg[4];
    elem_coords(m, e, x);
    global_grads(x, dim, gg);
    const int* ev = m->elem_verts + (size_t)e * nn;
    if (ncomp_in == 1) {
      /* ScalarElement::grad (apf/apfScalarElement.cc:18) */
      V3 g = v3_scale(gg[0], f[ev[0]]);
      for (int i = 1; i < nn; ++i) g = v3_add(g, v3_scale(gg[i], f[ev[i]]));
      for (int k = 0; k < 3; ++k) ip[(size_t)e * 3 + k] = g.v[k];
    } else {
      /* VectorElement::grad -> gradHelper: g = sum tensorProduct(gg_i, u_i) */
      M3 g;
      for (int i = 0; i < nn; ++i) {
        V3 u = {{f[3 * ev[i]], f[3 * ev[i] + 1], f[3 * ev[i] + 2]}};
        for (int r = 0; r < 3; ++r) {
          V3 row = v3_scale(u, gg[i].v[r]);
          if (i == 0) m3_setrow(&g, r, row);
          else m3_setrow(&g, r, v3_add(m3_row(g, r), row));
        }
      }
      for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) ip[(size_t)e * 9 + 3 * r + c] = g.m[r][c];
    }
  }
  return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* mth Householder QR (mth/mthQR.cc:19-160)                             */
/* A, R: m x n row-major; Q: m x m row-major                            */
/* ------------------------------------------------------------------ */
static double sgn(double x) { return (x < 0) ? -1 : 1; }

static int get_reflector(const double* a, int m, int n, double* v, int k) {
  double cnorm = 0;
  for (int i = k; i < m; ++i) cnorm += a[i * n + k] * a[i * n + k];
  cnorm = sqrt(cnorm);
  if (cnorm < 1e-10) return 0;
  for (int i = 0; i < k; ++i) v[i] = 0;
  for (int i = k; i < m; ++i) v[i] = a[i * n + k];
  v[k] += sgn(a[k * n + k]) * cnorm;
  double rnorm = 0;
  for (int i = k; i < m; ++i) rnorm += v[i] * v[i];
  rnorm = sqrt(rnorm);
  for (int i = k; i < m; ++i) v[i] /= rnorm;
  return 1;
}

int orc_qr_decompose(int m, int n, const double* A, double* Q, double* R, double* vscratch) {
  for (int i = 0; i < m; ++i) for (int j = 0; j < m; ++j) Q[i * m + j] = (double)(i == j);
  memcpy(R, A, sizeof(double) * (size_t)m * n);
  int rank = 0;
  for (int k = 0; k < n; ++k) {
    if (!get_reflector(R, m, n, vscratch, k)) continue;
    /* reflect_columns */
    for (int j = 0; j < n; ++j) {
      double dot = 0;
      for (int i = k; i < m; ++i) dot += R[i * n + j] * vscratch[i];
      for (int i = k; i < m; ++i) R[i * n + j] -= 2 * dot * vscratch[i];
    }
    /* reflect_rows */
    for (int i = 0; i < m; ++i) {
      double dot = 0;
      for (int j = k; j < m; ++j) dot += Q[i * m + j] * vscratch[j];
      for (int j = k; j < m; ++j) Q[i * m + j] -= 2 * dot * vscratch[j];
    }
    ++rank;
  }
  return rank;
}

/* solveFromQR: y = transpose(Q) b (full m), backsubUT (mth/mthQR.cc:132-160) */
void orc_qr_solve_from(int m, int n, const double* Q, const double* R, const double* b, double* x, double* y) {
  for (int i = 0; i < m; ++i) {
    y[i] = 0;
    for (int j = 0; j < m; ++j) y[i] += Q[j * m + i] * b[j];
  }
  for (int ii = 0; ii < n; ++ii) {
    int i = n - ii - 1;
    x[i] = y[i];
    for (int j = i + 1; j < n; ++j) x[i] -= R[i * n + j] * x[j];
    x[i] /= R[i * n + i];
  }
}

/* mth::solveQR: returns rank; x valid iff rank == n */
int orc_qr_solve(int m, int n, const double* A, const double* b, double* x) {
  double* Q = (double*)malloc(sizeof(double) * (size_t)m * m);
  double* R = (double*)malloc(sizeof(double) * (size_t)m * n);
  double* v = (double*)malloc(sizeof(double) * (size_t)m);
  double* y = (double*)malloc(sizeof(double) * (size_t)m);
  int rank = orc_qr_decompose(m, n, A, Q, R, v);
  if (rank == n) orc_qr_solve_from(m, n, Q, R, b, x, y);
  free(Q); free(R); free(v); free(y);
  return rank;
}

/* ------------------------------------------------------------------ */
/* spr::recoverField (spr/sprRecoverField.cc), linear mesh              */
/* ------------------------------------------------------------------ */
typedef struct {
  int* el; int n, cap;          /* patch element set, ascending index */
  int* mark; int mark_gen;      /* per-element membership stamp (size T) */
  int* old; int nold;
  double *A, *Q, *R, *v, *y, *b, *c;
  int qcap;
} patch_ws;

static void ws_reserve(patch_ws* w, int m) {
  if (m <= w->qcap) return;
  int cap = m * 2;
  w->A = (double*)realloc(w->A, sizeof(double) * (size_t)cap * 4);
  w->R = (double*)realloc(w->R, sizeof(double) * (size_t)cap * 4);
  w->Q = (double*)realloc(w->Q, sizeof(double) * (size_t)cap * cap);
  w->v = (double*)realloc(w->v, sizeof(double) * (size_t)cap);
  w->y = (double*)realloc(w->y, sizeof(double) * (size_t)cap);
  w->b = (double*)realloc(w->b, sizeof(double) * (size_t)cap);
  w->qcap = cap;
}

static int cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

static void patch_add(patch_ws* w, int e) {
  if (w->mark[e] == w->mark_gen) return;
  w->mark[e] = w->mark_gen;
  if (w->n == w->cap) { w->cap = w->cap ? 2 * w->cap : 64; w->el = (int*)realloc(w->el, sizeof(int) * w->cap); }
  w->el[w->n++] = e;
}

/* hasEnoughPoints -> prepareSpr -> preparePolynomialFit (spr/sprRecoverField.cc:283-362) */
static int patch_ready(const orc_mesh* m, patch_ws* w, int nterms) {
  if (w->n < nterms) return 0; /* one point per element */
  qsort(w->el, w->n, sizeof(int), cmp_int); /* std::set<MeshEntity*> order = ascending id */
  int mm = w->n, dim = m->dim;
  ws_reserve(w, mm);
  V3 xi = ip_point(dim);
  double N[4];
  shape_values(dim, xi, N);
  for (int i = 0; i < mm; ++i) {
    V3 x[4];
    elem_coords(m, w->el[i], x);
    double nodes[12], p[3];
    for (int a = 0; a < dim + 1; ++a) for (int k = 0; k < 3; ++k) nodes[3 * a + k] = x[a].v[k];
    interp(nodes, dim + 1, 3, N, p); /* mapLocalToGlobal */
    w->A[i * nterms + 0] = 1.0;
    w->A[i * nterms + 1] = p[0];
    w->A[i * nterms + 2] = p[1];
    if (nterms == 4) w->A[i * nterms + 3] = p[2];
  }
  int rank = orc_qr_decompose(mm, nterms, w->A, w->Q, w->R, w->v);
  return rank == nterms;
}

/* elements sharing a dimension-sd entity with the set `old`
   (addElementsThatShare, spr/sprRecoverField.cc:165-187).  In a conforming
   simplicial mesh two elements share an sd-entity iff they share sd+1
   vertices. */
static void add_sharing(const orc_mesh* m, patch_ws* w, int sd) {
  int nv = m->dim + 1;
  for (int i = 0; i < w->nold; ++i) {
    int e = w->old[i];
    const int* ev = m->elem_verts + (size_t)e * nv;
    for (int a = 0; a < nv; ++a) {
      int v = ev[a];
      for (int k = m->v2e_off[v]; k < m->v2e_off[v + 1]; ++k) {
        int f = m->v2e[k];
        if (w->mark[f] == w->mark_gen) continue;
        const int* fv = m->elem_verts + (size_t)f * nv;
        int shared = 0;
        for (int p = 0; p < nv; ++p) for (int q = 0; q < nv; ++q) if (ev[p] == fv[q]) ++shared;
        if (shared >= sd + 1) patch_add(w, f);
      }
    }
  }
}

/* expandAsNecessary (spr/sprRecoverField.cc:365-386); returns 0 on failure */
static int build_patch(const orc_mesh* m, patch_ws* w, int v, int nterms, int* expanded) {
  w->mark_gen++;
  w->n = 0;
  for (int k = m->v2e_off[v]; k < m->v2e_off[v + 1]; ++k) patch_add(w, m->v2e[k]);
  *expanded = 0;
  for (;;) {
    if (patch_ready(m, w, nterms)) return 1;
    *expanded = 1;
    if (w->nold < w->n) w->old = (int*)realloc(w->old, sizeof(int) * (size_t)w->n);
    memcpy(w->old, w->el, sizeof(int) * (size_t)w->n);
    w->nold = w->n;
    for (int sd = m->dim - 1; sd >= 0; --sd) {
      add_sharing(m, w, sd);
      if (patch_ready(m, w, nterms)) return 1;
    }
    if (!(w->n > w->nold)) return 0; /* "all hope is lost" */
  }
}

/* runSpr (spr/sprRecoverField.cc:327-353) */
static void run_spr(const orc_mesh* m, patch_ws* w, int v, const double* ip, int nc, int nterms, double* out) {
  int mm = w->n;
  V3 xv = vert_xyz(m, v);
  double terms[4] = {1.0, xv.v[0], xv.v[1], xv.v[2]};
  double coeffs[4];
  for (int i = 0; i < nc; ++i) {
    for (int j = 0; j < mm; ++j) w->b[j] = ip[(size_t)w->el[j] * nc + i];
    orc_qr_solve_from(mm, nterms, w->Q, w->R, w->b, coeffs, w->y);
    double s = 0;
    for (int j = 0; j < nterms; ++j) s += coeffs[j] * terms[j];
    out[(size_t)v * nc + i] = s;
  }
}

/* Returns ORC_EPATCH if a patch cannot be completed; *n_expanded counts
   vertices whose initial patch had to grow; fail_vertex gets the first bad one. */
int orc_recover(const orc_mesh* m, const double* ip, int nc, double* out, int* n_expanded, int* fail_vertex) {
  int nterms = m->dim == 3 ? 4 : 3;
  int V = m->n[0], T = m->n[m->dim];
  int nexp = 0, fail = -1;
#pragma omp parallel
  {
    patch_ws w;
    memset(&w, 0, sizeof w);
    w.mark = (int*)calloc((size_t)T, sizeof(int));
    int my_exp = 0;
#pragma omp for schedule(dynamic, 256)
    for (int v = 0; v < V; ++v) {
      int expanded = 0;
      if (!build_patch(m, &w, v, nterms, &expanded)) {
#pragma omp critical
        { if (fail < 0 || v < fail) fail = v; }
        continue;
      }
      my_exp += expanded;
      run_spr(m, &w, v, ip, nc, nterms, out);
    }
#pragma omp atomic
    nexp += my_exp;
    free(w.el); free(w.mark); free(w.old); free(w.A); free(w.Q); free(w.R); free(w.v); free(w.y); free(w.b);
  }
  if (n_expanded) *n_expanded = nexp;
  if (fail_vertex) *fail_vertex = fail;
  return fail >= 0 ? ORC_EPATCH : ORC_OK;
}

/* ------------------------------------------------------------------ */
/* spr::getSPRSizeField (spr/sprEstimateError.cc) and                  */
/* spr::getTargetSPRSizeField (spr/sprEstimateTargetError.cc)           */
/* ------------------------------------------------------------------ */

/* apf::measure on a linear edge: N1 rule, w = 2 (apf/apfIntegrate.cc:689-702) */
static double edge_measure(V3 x0, V3 x1) {
  V3 x[2] = {x0, x1};
  M3 J = jacobian(x, 2, 1);
  double dV = jacobian_det(J, 1);
  double r = 0;
  r += 2 * dV;
  return r;
}

/* getCurrentSize: max over downward edges of apf::measure (spr/sprEstimateError.cc:219) */
static double current_size(const orc_mesh* m, int e) {
  int ne = m->dim == 3 ? 6 : 3;
  const int* ee = m->elem_edges + (size_t)e * ne;
  double h = 0;
  for (int i = 0; i < ne; ++i) {
    const int* ev = m->dn[1] + 2 * (size_t)ee[i];
    double l = edge_measure(vert_xyz(m, ev[0]), vert_xyz(m, ev[1]));
    h = (h < l) ? l : h; /* std::max */
  }
  return h;
}

/* per element: eps* interpolated at the IP; SelfProduct term and the
   ElementError sum (spr/sprEstimateError.cc:98-170) */
static void element_terms(const orc_mesh* m, int e, const double* ip, const double* rec, int nc,
                          double* self_term, double* err_sum) {
  int dim = m->dim, nn = dim + 1;
  V3 x[4];
  elem_coords(m, e, x);
  V3 xi = ip_point(dim);
  double w = ip_weight(dim);
  M3 J = jacobian(x, nn, dim);
  double dV = jacobian_det(J, dim);
  double N[4];
  shape_values(dim, xi, N);
  double nodes[4 * 9], v2[9], v1[9];
  const int* ev = m->elem_verts + (size_t)e * nn;
  for (int a = 0; a < nn; ++a)
    for (int k = 0; k < nc; ++k) nodes[a * nc + k] = rec[(size_t)ev[a] * nc + k];
  interp(nodes, nn, nc, N, v2);
  double vv = 0;
  for (int k = 0; k < nc; ++k) vv += v2[k] * v2[k];
  *self_term = vv * w * dV;
  for (int k = 0; k < nc; ++k) v1[k] = ip[(size_t)e * nc + k];
  for (int k = 0; k < nc; ++k) v1[k] -= v2[k];
  double dd = 0;
  for (int k = 0; k < nc; ++k) dd += v1[k] * v1[k];
  double sum = 0;
  sum += dd * w * dV;
  *err_sum = sum;
}

typedef struct {
  double eps_star_norm2;  /* SelfProduct result */
  double error_sum;       /* Error / GlobalErrorTerm result */
  double size_factor;
  int n_expanded;
  int fail_vertex;
} orc_size_info;

/* averageSizeField: mean over getAdjacent(v, dim) in MDS order (spr/sprEstimateError.cc:255) */
static void average_to_vertex(const orc_mesh* m, const double* esize, double* size) {
  int V = m->n[0];
#pragma omp parallel for schedule(static)
  for (int v = 0; v < V; ++v) {
    double s = 0;
    int b = m->v2e_off[v], e = m->v2e_off[v + 1];
    for (int k = b; k < e; ++k) s += esize[m->v2e[k]];
    s /= (double)(size_t)(e - b);
    size[v] = s;
  }
}

/* mode 0: getSPRSizeField(eps, adapt_ratio); mode 1: getTargetSPRSizeField(eps, target, alpha, beta).
   rec_out (V x nc), esize_out (T), err_out (T): optional intermediates. */
int orc_size_field(const orc_mesh* m, const double* ip, int nc, int mode, double adapt_ratio,
                   double target, double alpha, double beta,
                   double* size_out, double* rec_out, double* esize_out, double* err_out, orc_size_info* info) {
  int dim = m->dim, V = m->n[0], T = m->n[dim];
  double* rec = rec_out ? rec_out : (double*)malloc(sizeof(double) * (size_t)V * nc);
  double* self = (double*)malloc(sizeof(double) * (size_t)T);
  double* errs = (double*)malloc(sizeof(double) * (size_t)T);
  double* esize = esize_out ? esize_out : (double*)malloc(sizeof(double) * (size_t)T);
  int nexp = 0, failv = -1;
  int rc = orc_recover(m, ip, nc, rec, &nexp, &failv);
  if (info) { info->n_expanded = nexp; info->fail_vertex = failv; }
  if (rc) goto done;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < T; ++e) element_terms(m, e, ip, rec, nc, &self[e], &errs[e]);
  double d = dim, p = 1; /* recovered order = mesh order = 1 */
  double snorm = 0, gsum = 0, size_factor;
  if (mode == 0) {
    /* computeSizeFactor: two sequential integrator sweeps in element order */
    for (int e = 0; e < T; ++e) snorm += self[e];
    for (int e = 0; e < T; ++e) gsum += pow(sqrt(errs[e]), ((2 * d) / (2 * p + d)));
    double esn = sqrt(snorm);
    double a = adapt_ratio * adapt_ratio * esn * esn;
    double b = a / gsum;
    size_factor = pow(b, 1.0 / (2.0 * p));
  } else {
    for (int e = 0; e < T; ++e) gsum += pow(sqrt(errs[e]), ((2 * d) / (2 * p + d)));
    double N = target;
    size_factor = pow((gsum / N), (1.0 / dim));
  }
  if (info) { info->eps_star_norm2 = snorm; info->error_sum = gsum; info->size_factor = size_factor; }
#pragma omp parallel for schedule(static)
  for (int e = 0; e < T; ++e) {
    double h = current_size(m, e);
    if (mode == 0) {
      /* getDesiredSize (spr/sprEstimateError.cc:230) */
      double errorNorm = pow(sqrt(errs[e]), -(2 / (2 * p + d)));
      esize[e] = h * errorNorm * size_factor;
    } else {
      /* getNewSize (spr/sprEstimateTargetError.cc:149) */
      int pi = 1, di = dim;
      double theta_e = sqrt(errs[e]);
      double r = pow(theta_e, ((-2.0) / (2.0 * pi + di)));
      double h_new = size_factor * r * h;
      if (h_new < alpha * h) h_new = alpha * h;
      if (h_new > beta * h) h_new = beta * h;
      esize[e] = h_new;
    }
  }
  if (err_out) memcpy(err_out, errs, sizeof(double) * (size_t)T);
  average_to_vertex(m, esize, size_out);
done:
  if (!rec_out) free(rec);
  if (!esize_out) free(esize);
  free(self); free(errs);
  return rc;
}

/* ------------------------------------------------------------------ */
/* ma size field transform, metric length, marks, quality              */
/* ------------------------------------------------------------------ */

/* orthogonalizeR (ma/maSize.cc:94-117) */
static M3 orthogonalize(M3 R) {
  M3 RT = m3_transpose(R);
  V3 r0 = v3_normalize(m3_row(RT, 0));
  V3 r1 = m3_row(RT, 1);
  r1 = v3_sub(r1, v3_scale(r0, v3_dot(r0, r1)));
  r1 = v3_normalize(r1);
  V3 r2 = v3_cross(r0, r1);
  m3_setrow(&RT, 0, r0); m3_setrow(&RT, 1, r1); m3_setrow(&RT, 2, r2);
  return m3_transpose(RT);
}

/* AnisoSizeField::getTransform (ma/maSize.cc:395-412): h and R interpolated
   with linear Lagrange shape values N over nn nodes.  hv: nn x 3, Rv: nn x 9
   (row-major) or NULL for identity frames (IsoWrapper). */
static M3 get_transform(const double* hv, const double* Rv, const double* N, int nn) {
  double h[3], R9[9];
  interp(hv, nn, 3, N, h);
  if (Rv) interp(Rv, nn, 9, N, R9);
  else {
    double I9[3 * 9];
    for (int a = 0; a < nn; ++a)
      for (int k = 0; k < 9; ++k) I9[a * 9 + k] = (k % 4 == 0) ? 1.0 : 0.0;
    interp(I9, nn, 9, N, R9);
  }
  M3 R;
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) R.m[i][j] = R9[3 * i + j];
  R = orthogonalize(R);
  M3 S;
  memset(&S, 0, sizeof S);
  S.m[0][0] = 1 / h[0]; S.m[1][1] = 1 / h[1]; S.m[2][2] = 1 / h[2];
  return m3_mul(R, S);
}

/* ------------------------------------------------------------------ */
/* mth::eigenQR for 3x3 (mth/mthQR.cc:19-297) and apf::eigen            */
/* (apf/apfMatrix.cc:68-82): Hessenberg reduction, Wilkinson-shifted QR */
/* with deflation from the bottom, at most max_iters steps              */
/* ------------------------------------------------------------------ */
typedef struct { double a[3][3]; } Q3;

static void q3_identity(Q3* q) {
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) q->a[i][j] = (double)(i == j);
}
/* get_reflector with offset o (mth/mthQR.cc:19-45) */
static int q3_reflector(const Q3* a, double v[3], int k, int o) {
  double cnorm = 0;
  for (int i = k + o; i < 3; ++i) cnorm += a->a[i][k] * a->a[i][k];
  cnorm = sqrt(cnorm);
  if (cnorm < 1e-10) return 0;
  for (int i = 0; i < k + o; ++i) v[i] = 0;
  for (int i = k + o; i < 3; ++i) v[i] = a->a[i][k];
  v[k + o] += sgn(a->a[k + o][k]) * cnorm;
  double rnorm = 0;
  for (int i = k + o; i < 3; ++i) rnorm += v[i] * v[i];
  rnorm = sqrt(rnorm);
  for (int i = k + o; i < 3; ++i) v[i] /= rnorm;
  return 1;
}
/* reflect_columns / reflect_rows (mth/mthQR.cc:47-79) */
static void q3_reflect_columns(const double v[3], Q3* a, int k, int o) {
  for (int j = 0; j < 3; ++j) {
    double dot = 0;
    for (int i = k + o; i < 3; ++i) dot += a->a[i][j] * v[i];
    for (int i = k + o; i < 3; ++i) a->a[i][j] -= 2 * dot * v[i];
  }
}
static void q3_reflect_rows(const double v[3], Q3* q, int k, int o) {
  for (int i = 0; i < 3; ++i) {
    double dot = 0;
    for (int j = k + o; j < 3; ++j) dot += q->a[i][j] * v[j];
    for (int j = k + o; j < 3; ++j) q->a[i][j] -= 2 * dot * v[j];
  }
}
/* mth::multiply (mth/mth_def.h:235-248): c(i,j) = 0, += a(i,l) b(l,j) */
static void q3_mul(const Q3* a, const Q3* b, Q3* c) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      c->a[i][j] = 0;
      for (int l = 0; l < 3; ++l) c->a[i][j] += a->a[i][l] * b->a[l][j];
    }
}
int orc_eigen_qr3(const double* A9, double* L9, double* Q9, int max_iters) {
  Q3 a, q, h, rk, qk, tmp;
  double v[3];
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) a.a[i][j] = A9[3 * i + j];
  /* reduceToHessenberg (mth/mthQR.cc:192-209) */
  q3_identity(&q);
  h = a;
  if (q3_reflector(&h, v, 0, 1)) {
    q3_reflect_columns(v, &h, 0, 1);
    q3_reflect_rows(v, &h, 0, 1);
    q3_reflect_rows(v, &q, 0, 1);
  }
  int red_m = 3, converged = 0;
  for (int it = 0; it < max_iters; ++it) {
    /* reduce (mth/mthQR.cc:211-222) */
    int more = 0;
    while (red_m > 1) {
      if (fabs(h.a[red_m - 2][red_m - 1]) < 1e-10 && fabs(h.a[red_m - 1][red_m - 2]) < 1e-10) --red_m;
      else { more = 1; break; }
    }
    if (!more) { converged = 1; break; }
    /* get_wilkinson_shift (mth/mthQR.cc:224-236) */
    double amm1 = h.a[red_m - 2][red_m - 2], am = h.a[red_m - 1][red_m - 1], bmm1 = h.a[red_m - 2][red_m - 1];
    double sig = (amm1 - am) / 2;
    double denom = (fabs(sig) + sqrt(sig * sig + bmm1 * bmm1));
    if (!(fabs(denom) > 1e-10)) return -1; /* PCU_ALWAYS_ASSERT */
    double mu = am - ((sgn(sig) * (bmm1 * bmm1)) / denom);
    for (int i = 0; i < 3; ++i) h.a[i][i] -= mu;
    /* decomposeQR (mth/mthQR.cc:106-126) */
    q3_identity(&qk);
    rk = h;
    for (int k = 0; k < 3; ++k)
      if (q3_reflector(&rk, v, k, 0)) {
        q3_reflect_columns(v, &rk, k, 0);
        q3_reflect_rows(v, &qk, k, 0);
      }
    q3_mul(&rk, &qk, &h);
    for (int i = 0; i < 3; ++i) h.a[i][i] -= -mu;
    q3_mul(&q, &qk, &tmp);
    q = tmp;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) { L9[3 * i + j] = h.a[i][j]; Q9[3 * i + j] = q.a[i][j]; }
  return converged;
}

/* LogAnisoSizeField::getTransform (ma/maSize.cc:508-523): logM interpolated
   over nn nodes (Mv: nn x 9), apf::eigen + orthogonalEigenDecompForSymmetric
   Matrix (ma/maSize.cc:123-142), Q = R diag(sqrt(exp(v))).  *ok = 0 when the
   eigen iteration fails (the reference asserts). */
static M3 log_transform(const double* Mv, const double* N, int nn, int* ok) {
  double M9[9], L9[9], Q9[9];
  interp(Mv, nn, 9, N, M9);
  if (orc_eigen_qr3(M9, L9, Q9, 100) != 1) *ok = 0;
  double val[3];
  V3 vec[3];
  for (int i = 0; i < 3; ++i) val[i] = L9[4 * i];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) vec[j].v[i] = Q9[3 * i + j];
  V3 r0 = v3_normalize(vec[0]);
  V3 r1 = v3_sub(vec[1], v3_scale(r0, v3_dot(r0, vec[1])));
  r1 = v3_normalize(r1);
  V3 r2 = v3_cross(r0, r1);
  M3 RT;
  m3_setrow(&RT, 0, r0); m3_setrow(&RT, 1, r1); m3_setrow(&RT, 2, r2);
  M3 R = m3_transpose(RT);
  M3 S;
  memset(&S, 0, sizeof S);
  S.m[0][0] = sqrt(exp(val[0])); S.m[1][1] = sqrt(exp(val[1])); S.m[2][2] = sqrt(exp(val[2]));
  return m3_mul(R, S);
}

/* LogAnisoSizeField::init (ma/maSize.cc:472-503): logM = f diag(log(1/h/h)) f^T */
static void vertex_logm(const double* sizes3, const double* frames9, int v, double* out9) {
  const double* h = sizes3 + 3 * (size_t)v;
  M3 f, S;
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) f.m[i][j] = frames9[9 * (size_t)v + 3 * i + j];
  memset(&S, 0, sizeof S);
  S.m[0][0] = log(1 / h[0] / h[0]); S.m[1][1] = log(1 / h[1] / h[1]); S.m[2][2] = log(1 / h[2] / h[2]);
  M3 r = m3_mul(m3_mul(f, S), m3_transpose(f));
  for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) out9[3 * i + j] = r.m[i][j];
}

int orc_log_metric(const orc_mesh* m, const double* sizes3, const double* frames9, double* logm9) {
  for (int v = 0; v < m->n[0]; ++v) vertex_logm(sizes3, frames9, v, logm9 + 9 * (size_t)v);
  return ORC_OK;
}

static void vertex_metric(const double* sizes3, const double* frames9, const double* size1, int v,
                          double* hv, double* Rv) {
  if (size1) { hv[0] = hv[1] = hv[2] = size1[v]; }
  else { for (int k = 0; k < 3; ++k) hv[k] = sizes3[3 * (size_t)v + k]; }
  if (Rv) {
    if (frames9) for (int k = 0; k < 9; ++k) Rv[k] = frames9[9 * (size_t)v + k];
    else for (int k = 0; k < 9; ++k) Rv[k] = (k % 4 == 0) ? 1.0 : 0.0;
  }
}

/* MetricSizeField::measure with SizeFieldIntegrator order 2: two Gauss points
   +-0.577350269189626, w = 1 (ma/maSize.cc:158-214, apf/apfIntegrate.cc:41-53).
   Either size1 (IsoUserField: makeSizeField(m, size)) or sizes3 + frames9
   (AnisoSizeField::init: makeSizeField(m, sizes, frames, false)). */
/* MetricSizeField::measure of the vertex pair (a, b) (ma/maSize.cc:158-216) */
static int g_log_ok = 1; /* cleared when an eigen iteration of a log-metric transform fails */

static double pair_metric_length_mode(const orc_mesh* m, int a0, int b0, const double* size1, const double* sizes3,
                                      const double* frames9, int logi) {
  const int ev[2] = {a0, b0};
  V3 x[2] = {vert_xyz(m, ev[0]), vert_xyz(m, ev[1])};
  double hv[6], Rv[18], Mv[18];
  for (int a = 0; a < 2; ++a) {
    if (logi) vertex_logm(sizes3, frames9, ev[a], Mv + 9 * a);
    else vertex_metric(sizes3, frames9, size1, ev[a], hv + 3 * a, Rv + 9 * a);
  }
  static const double gp[2] = {0.577350269189626, -0.577350269189626};
  M3 J = jacobian(x, 2, 1);
  double measurement = 0;
  for (int p = 0; p < 2; ++p) {
    V3 xi = {{gp[p], 0, 0}};
    double N[2];
    shape_values(1, xi, N);
    int ok = 1;
    M3 Q = logi ? log_transform(Mv, N, 2, &ok) : get_transform(hv, Rv, N, 2);
    if (!ok) g_log_ok = 0;
    double dV2 = jacobian_det(m3_mul(J, Q), 1);
    measurement += 1 * dV2;
  }
  return measurement;
}

static double pair_metric_length(const orc_mesh* m, int a0, int b0, const double* size1, const double* sizes3,
                                 const double* frames9) {
  return pair_metric_length_mode(m, a0, b0, size1, sizes3, frames9, 0);
}

static double metric_length(const orc_mesh* m, int edge, const double* size1, const double* sizes3, const double* frames9) {
  const int* ev = m->dn[1] + 2 * (size_t)edge;
  return pair_metric_length(m, ev[0], ev[1], size1, sizes3, frames9);
}

int orc_measure_edges(const orc_mesh* m, const double* size1, const double* sizes3, const double* frames9, double* L) {
  int E = m->n[1];
#pragma omp parallel for schedule(static)
  for (int e = 0; e < E; ++e) L[e] = metric_length(m, e, size1, sizes3, frames9);
  return ORC_OK;
}

/* markEntities (ma/maAdapt.cc:293-324) for edges with precomputed lengths.
   which 0: markEdgesToSplit (SPLIT, NEED_NOT_SPLIT, DONT_SPLIT|NEED_NOT_SPLIT, L > 1.5)
   which 1: markEdgesToCollapse (COLLAPSE, NEED_NOT_COLLAPSE, DONT_COLLAPSE|NEED_NOT_COLLAPSE, L < 0.5) */
int orc_mark_edges(int E, const double* L, int which, int* flags, long* count) {
  const int SPLIT = 1 << 0, DONT_SPLIT = 1 << 1, COLLAPSE = 1 << 2, DONT_COLLAPSE = 1 << 3;
  const int NEED_NOT_SPLIT = 1 << 17, NEED_NOT_COLLAPSE = 1 << 18;
  int trueFlag = which == 0 ? SPLIT : COLLAPSE;
  int setFalse = which == 0 ? NEED_NOT_SPLIT : NEED_NOT_COLLAPSE;
  int allFalse = which == 0 ? (DONT_SPLIT | NEED_NOT_SPLIT) : (DONT_COLLAPSE | NEED_NOT_COLLAPSE);
  long c = 0;
  for (int e = 0; e < E; ++e)
    if (flags[e] & trueFlag) return ORC_EFLAGS; /* PCU_ALWAYS_ASSERT(!getFlag(trueFlag)) */
  for (int e = 0; e < E; ++e) {
    if (allFalse & flags[e]) continue;
    int pred = which == 0 ? (L[e] > 1.5) : (L[e] < .5);
    if (pred) { flags[e] |= trueFlag; ++c; }
    else flags[e] |= setFalse;
  }
  *count = c;
  return ORC_OK;
}

/* FixedMetricIntegrator qMeasure (ma/maQuality.cc:35-81), order 1 rules */
static double q_measure(const V3* x, int nn, int edim, M3 Q) {
  M3 J = jacobian(x, nn, edim);
  double w = edim == 3 ? 1.0 / 6.0 : (edim == 2 ? 1.0 / 2.0 : 2.0);
  double dV2 = jacobian_det(m3_mul(J, Q), edim);
  double measurement = 0;
  measurement += w * dV2;
  return measurement;
}

/* measureTetQuality / measureTriQuality with useMax = true (ma/maQuality.cc:83-167) */
static double element_quality_mode(const orc_mesh* m, int e, const double* size1, const double* sizes3,
                                   const double* frames9, int logi) {
  int dim = m->dim, nn = dim + 1;
  const int* ev = m->elem_verts + (size_t)e * nn;
  M3 Q;
  memset(&Q, 0, sizeof Q);
  double maxJ = -1.0;
  for (int i = 0; i < nn; ++i) {
    double hv[3], Rv[9], Mv[9], N[1] = {1.0};
    M3 cQ;
    if (logi) {
      int ok = 1;
      vertex_logm(sizes3, frames9, ev[i], Mv);
      cQ = log_transform(Mv, N, 1, &ok);
      if (!ok) g_log_ok = 0;
    } else {
      vertex_metric(sizes3, frames9, size1, ev[i], hv, Rv);
      cQ = get_transform(hv, Rv, N, 1);
    }
    double cJ = jacobian_det(cQ, dim);
    if (cJ > maxJ) { maxJ = cJ; Q = cQ; }
  }
  V3 x[4];
  elem_coords(m, e, x);
  int ne = dim == 3 ? 6 : 3;
  const int* ee = m->elem_edges + (size_t)e * ne;
  double s = 0;
  for (int i = 0; i < ne; ++i) {
    const int* evv = m->dn[1] + 2 * (size_t)ee[i];
    V3 xe[2] = {vert_xyz(m, evv[0]), vert_xyz(m, evv[1])};
    double l = q_measure(xe, 2, 1, Q);
    s += l * l;
  }
  double Vm = q_measure(x, nn, dim, Q);
  if (dim == 3) {
    if (Vm < 0) return -15552 * (Vm * Vm) / (s * s * s);
    return 15552 * (Vm * Vm) / (s * s * s);
  }
  return 48 * (Vm * Vm) / (s * s);
}

static double element_quality(const orc_mesh* m, int e, const double* size1, const double* sizes3, const double* frames9) {
  return element_quality_mode(m, e, size1, sizes3, frames9, 0);
}

/* makeSizeField(m, sizes, frames, true) (LogAnisoSizeField, ma/maSize.cc:455-580):
   metric lengths of every edge and qualities of every element.  Returns
   ORC_EEIGEN when an eigen iteration fails (the reference asserts). */
int orc_measure_edges_log(const orc_mesh* m, const double* sizes3, const double* frames9, double* L) {
  g_log_ok = 1;
  for (int e = 0; e < m->n[1]; ++e) {
    const int* ev = m->dn[1] + 2 * (size_t)e;
    L[e] = pair_metric_length_mode(m, ev[0], ev[1], NULL, sizes3, frames9, 1);
  }
  return g_log_ok ? ORC_OK : ORC_EEIGEN;
}

int orc_quality_log(const orc_mesh* m, const double* sizes3, const double* frames9, double* q) {
  g_log_ok = 1;
  for (int e = 0; e < m->n[m->dim]; ++e) q[e] = element_quality_mode(m, e, NULL, sizes3, frames9, 1);
  return g_log_ok ? ORC_OK : ORC_EEIGEN;
}

int orc_quality(const orc_mesh* m, const double* size1, const double* sizes3, const double* frames9, double* q) {
  int T = m->n[m->dim];
#pragma omp parallel for schedule(static)
  for (int e = 0; e < T; ++e) q[e] = element_quality(m, e, size1, sizes3, frames9);
  return ORC_OK;
}

/* whole estimate-and-mark pass on a scalar P1 field u (3D or 2D iso):
   getGradIPField(u,"grad",1) -> getSPRSizeField(grad, adapt_ratio) ->
   makeSizeField(m,size) -> measure every edge -> markEdgesToSplit and
   markEdgesToCollapse on fresh flags.  flags_out may be NULL. */
int orc_estimate_and_mark(const orc_mesh* m, const double* u, double adapt_ratio,
                          double* size_out, double* L_out, int* flags_out, long* n_split, long* n_collapse,
                          orc_size_info* info) {
  int dim = m->dim, T = m->n[dim], E = m->n[1];
  double* ip = (double*)malloc(sizeof(double) * (size_t)T * 3);
  double* L = L_out ? L_out : (double*)malloc(sizeof(double) * (size_t)E);
  int* flags = flags_out ? flags_out : (int*)calloc((size_t)E, sizeof(int));
  int rc = orc_grad_ip(m, u, 1, ip);
  if (!rc) rc = orc_size_field(m, ip, 3, 0, adapt_ratio, 0, 0, 0, size_out, NULL, NULL, NULL, info);
  if (!rc) rc = orc_measure_edges(m, size_out, NULL, NULL, L);
  if (!rc) {
    if (flags_out) memset(flags, 0, sizeof(int) * (size_t)E);
    long c1 = 0, c2 = 0;
    rc = orc_mark_edges(E, L, 0, flags, &c1);
    if (!rc) rc = orc_mark_edges(E, L, 1, flags, &c2);
    if (n_split) *n_split = c1;
    if (n_collapse) *n_collapse = c2;
  }
  free(ip);
  if (!L_out) free(L);
  if (!flags_out) free(flags);
  return rc;
}

/* ------------------------------------------------------------------ */
/* MA sweeps around the marks                                           */
/* ------------------------------------------------------------------ */
/* SizeField::measure of a vertex pair; kind 0: IdentitySizeField
   (apf::measure of the edge, ma/maSize.cc:54-60), 1: isotropic user field,
   2: anisotropic (sizes3, frames9), 3: LogAnisoSizeField of (sizes3, frames9) */
static double pair_length(const orc_mesh* m, int kind, int a, int b, const double* size1, const double* sizes3,
                          const double* frames9) {
  if (kind == 0) return edge_measure(vert_xyz(m, a), vert_xyz(m, b));
  if (kind == 3) return pair_metric_length_mode(m, a, b, NULL, sizes3, frames9, 1);
  return kind == 1 ? pair_metric_length(m, a, b, size1, NULL, NULL) : pair_metric_length(m, a, b, NULL, sizes3, frames9);
}

int orc_measure_pairs(const orc_mesh* m, int kind, const double* size1, const double* sizes3, const double* frames9,
                      long n, const int* pairs, double* L) {
  for (long i = 0; i < n; ++i) {
    if (pairs[2 * i] < 0 || pairs[2 * i] >= m->n[0] || pairs[2 * i + 1] < 0 || pairs[2 * i + 1] >= m->n[0])
      return ORC_EINVAL;
    L[i] = pair_length(m, kind, pairs[2 * i], pairs[2 * i + 1], size1, sizes3, frames9);
  }
  return ORC_OK;
}

/* getMaximumEdgeLength (ma/maSize.cc:673-690) */
double orc_max_edge_length(const orc_mesh* m, int kind, const double* size1, const double* sizes3,
                           const double* frames9) {
  double maxLength = 0.0;
  for (int e = 0; e < m->n[1]; ++e) {
    const int* ev = m->dn[1] + 2 * (size_t)e;
    double length = pair_length(m, kind, ev[0], ev[1], size1, sizes3, frames9);
    if (length > maxLength) maxLength = length;
  }
  return maxLength;
}

/* getAverageEdgeLength (ma/maSize.cc:652-671) */
double orc_average_edge_length(const orc_mesh* m) {
  double length_sum = 0, edge_count = 0;
  for (int e = 0; e < m->n[1]; ++e) {
    const int* ev = m->dn[1] + 2 * (size_t)e;
    length_sum += edge_measure(vert_xyz(m, ev[0]), vert_xyz(m, ev[1]));
    edge_count += 1.0;
  }
  return length_sum / edge_count;
}

/* updateMaxIterBasedOnSize (ma/maInput.cc:174-190) */
int orc_max_iterations(double max_metric_length) {
  int iter = (int)ceil(log2(max_metric_length));
  return iter >= 10 ? 10 : iter + 1;
}

/* markBadQuality = markEntities(dim, quality < goodQuality, BAD_QUALITY,
   OK_QUALITY) (ma/maShape.cc:132-136, ma/maAdapt.cc:293-324) */
int orc_mark_bad_quality(int T, const double* q, double good, int* flags, long* count) {
  const int BAD_QUALITY = 1 << 5, OK_QUALITY = 1 << 6;
  long c = 0;
  for (int e = 0; e < T; ++e)
    if (flags[e] & BAD_QUALITY) return ORC_EFLAGS;
  for (int e = 0; e < T; ++e) {
    if (OK_QUALITY & flags[e]) continue;
    if (q[e] < good) { flags[e] |= BAD_QUALITY; ++c; }
    else flags[e] |= OK_QUALITY;
  }
  *count = c;
  return ORC_OK;
}

/* getMinQuality (ma/maShape.cc:151-169) */
double orc_min_quality(int T, const double* q) {
  double minqual = 1;
  for (int e = 0; e < T; ++e)
    if (q[e] < minqual) minqual = q[e];
  return minqual;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}
