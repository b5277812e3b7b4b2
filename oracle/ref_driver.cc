// C entry points over the reference's own estimate-and-mark path -- TEST
// INFRASTRUCTURE ONLY.
//
// Linked against SCOREC/core's pcu, gmi, apf, mds, spr and ma compiled from
// their sources (oracle/Makefile, target refall) into oracle/_ref/libspr_ref.so.
// Every number these functions return is computed by the reference's code:
// apf::makeMdsBox / apf::loadMdsMesh for the mesh and its numbering,
// spr::getGradIPField, spr::recoverField, spr::getSPRSizeField /
// spr::getTargetSPRSizeField, ma::configure + ma::SizeField::measure,
// ma::markEdgesToCollapse / ma::markEdgesToSplit on an ma::Adapt, and
// ma::measureElementQuality.  The code here only moves values between flat
// arrays in MDS index order (apf::getMdsIndex) and apf fields, and times the
// calls.  The tests pin the oracle restatement (oracle/spr_oracle.c) and the
// GPU path to these outputs; bench.py can time this path as the reference's
// CPU baseline.
#include <apf.h>
#include <apfBox.h>
#include <apfMDS.h>
#include <apfMesh2.h>
#include <apfShape.h>
#include <gmi_mesh.h>
#include <gmi_null.h>
#include <lionPrint.h>
#include <ma.h>
#include <maAdapt.h>
#include <maCoarsen.h>
#include <maRefine.h>
#include <maShape.h>
#include <maSize.h>
#include <PCU.h>
#include <spr.h>

#include <chrono>
#include <cstring>
#include <vector>

namespace ma {
// defined in ma/maCoarsen.cc:287 without a header declaration
long markEdgesToCollapse(Adapt* a);
}

namespace {

pcu::PCU* the_pcu() {
  static pcu::PCU* p = nullptr;
  if (!p) {
    pcu::Init(nullptr, nullptr);
    lion_set_verbosity(0);
    p = new pcu::PCU();
    gmi_register_null();
    gmi_register_mesh();
  }
  return p;
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct RefMesh {
  apf::Mesh2* m = nullptr;
  int dim = 0;
  std::vector<apf::MeshEntity*> ents[4];  // by MDS index

  void index() {
    dim = m->getDimension();
    for (int d = 0; d <= dim; ++d) {
      ents[d].assign(m->count(d), nullptr);
      apf::MeshIterator* it = m->begin(d);
      apf::MeshEntity* e;
      while ((e = m->iterate(it))) ents[d][apf::getMdsIndex(m, e)] = e;
      m->end(it);
    }
  }
  int idx(apf::MeshEntity* e) { return apf::getMdsIndex(m, e); }
};

apf::Field* make_vertex_field(RefMesh* r, const char* name, int type, const double* vals) {
  apf::Field* f = apf::createFieldOn(r->m, name, type);
  const int nc = apf::countComponents(f);
  for (size_t i = 0; i < r->ents[0].size(); ++i) apf::setComponents(f, r->ents[0][i], 0, vals + nc * i);
  return f;
}

// ma::configure on the given size field(s), an ma::Adapt over it, and the
// collapse pass then the split pass of markEntities (the order ma::adapt
// runs coarsen and refine, ma/ma.cc); lengths, flags and qualities read back
int mark_with(RefMesh* r, const ma::Input* cin, double* lengths, int* flags, long* n_split, long* n_collapse,
              double* quality, double* seconds) {
  ma::Input* in = ma::makeAdvanced(cin);
  double t0 = now();
  ma::Adapt* a = new ma::Adapt(in);
  const long nc = ma::markEdgesToCollapse(a);
  const long ns = ma::markEdgesToSplit(a);
  double t1 = now();
  ma::SizeField* sf = in->sizeField;
  for (size_t i = 0; i < r->ents[1].size(); ++i) {
    if (lengths) lengths[i] = sf->measure(r->ents[1][i]);
    if (flags) flags[i] = ma::getFlags(a, r->ents[1][i]);
  }
  double t2 = now();
  if (quality)
    for (size_t i = 0; i < r->ents[r->dim].size(); ++i)
      quality[i] = ma::measureElementQuality(r->m, sf, r->ents[r->dim][i]);
  double t3 = now();
  if (n_split) *n_split = ns;
  if (n_collapse) *n_collapse = nc;
  if (seconds) {
    seconds[0] = t1 - t0;  // Adapt set-up + both marking passes
    seconds[1] = t2 - t1;  // measure of every edge (read-back)
    seconds[2] = t3 - t2;  // quality of every element
  }
  delete a;
  if (in->ownsSolutionTransfer) delete in->solutionTransfer;
  delete in->sizeField;
  delete in;
  return 0;
}

}  // namespace

extern "C" {

void* refd_box(int nx, int ny, int nz) {
  RefMesh* r = new RefMesh;
  r->m = apf::makeMdsBox(nx, ny, nz, 1, 1, nz ? 1 : 0, true, the_pcu());
  r->index();
  return r;
}

// a .smb mesh on the null model (mesh entities classified on model entities
// the null model creates as they are looked up); smb names the file without
// its part number ("mesh.smb" reads mesh0.smb), as apf::loadMdsMesh takes it
void* refd_load(const char* smb) {
  RefMesh* r = new RefMesh;
  gmi_model* g = (the_pcu(), gmi_load(".null"));
  r->m = apf::loadMdsMesh(g, smb, the_pcu());
  r->index();
  return r;
}

void refd_free(void* h) {
  RefMesh* r = (RefMesh*)h;
  if (!r) return;
  r->m->destroyNative();
  apf::destroyMesh(r->m);
  delete r;
}

int refd_dim(void* h) { return ((RefMesh*)h)->dim; }
long refd_count(void* h, int d) { return (long)((RefMesh*)h)->ents[d].size(); }

// the reference's numbering: coordinates, element vertices (getDownward(e, 0))
// and edge vertices, all in MDS index order
void refd_mesh(void* h, double* coords, int* elem_verts, int* edge_verts) {
  RefMesh* r = (RefMesh*)h;
  for (size_t i = 0; i < r->ents[0].size(); ++i) {
    apf::Vector3 p;
    r->m->getPoint(r->ents[0][i], 0, p);
    for (int k = 0; k < 3; ++k) coords[3 * i + k] = p[k];
  }
  apf::Downward dv;
  const int nv = r->dim + 1;
  for (size_t i = 0; i < r->ents[r->dim].size(); ++i) {
    r->m->getDownward(r->ents[r->dim][i], 0, dv);
    for (int k = 0; k < nv; ++k) elem_verts[nv * i + k] = r->idx(dv[k]);
  }
  for (size_t i = 0; i < r->ents[1].size(); ++i) {
    r->m->getDownward(r->ents[1][i], 0, dv);
    edge_verts[2 * i] = r->idx(dv[0]);
    edge_verts[2 * i + 1] = r->idx(dv[1]);
  }
}

// getAdjacent(v, dim) of every vertex, in the order the reference returns it
// (CSR: off n_verts + 1, adj off[n_verts])
void refd_vert_elems(void* h, int* off, int* adj) {
  RefMesh* r = (RefMesh*)h;
  int k = 0;
  for (size_t i = 0; i < r->ents[0].size(); ++i) {
    off[i] = k;
    apf::Adjacent a;
    r->m->getAdjacent(r->ents[0][i], r->dim, a);
    for (size_t j = 0; j < a.getSize(); ++j) adj[k++] = r->idx(a[j]);
  }
  off[r->ents[0].size()] = k;
}

void refd_set_coords(void* h, const double* coords) {
  RefMesh* r = (RefMesh*)h;
  for (size_t i = 0; i < r->ents[0].size(); ++i)
    r->m->setPoint(r->ents[0][i], 0, apf::Vector3(coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]));
}

// spr::getGradIPField(u, "grad", 1) of the scalar vertex field u, then
// (each output may be NULL) the IP values ip_out (n_elems x 3),
// spr::recoverField of them rec_out (n_verts x 3), and
//   mode 0: spr::getSPRSizeField(grad, adapt_ratio)
//   mode 1: spr::getTargetSPRSizeField(grad, target, alpha, beta)
// size_out (n_verts).  seconds[0..2]: gradient, recovery, size field.
int refd_spr(void* h, const double* u, int mode, double adapt_ratio, long target, double alpha, double beta,
             double* ip_out, double* rec_out, double* size_out, double* seconds) {
  RefMesh* r = (RefMesh*)h;
  apf::Field* uf = make_vertex_field(r, "refd_u", apf::SCALAR, u);
  double t0 = now();
  apf::Field* grad = spr::getGradIPField(uf, "grad", 1);
  double t1 = now();
  if (ip_out)
    for (size_t i = 0; i < r->ents[r->dim].size(); ++i) {
      apf::Vector3 g;
      apf::getVector(grad, r->ents[r->dim][i], 0, g);
      for (int k = 0; k < 3; ++k) ip_out[3 * i + k] = g[k];
    }
  double t2 = t1, t3 = t1;
  if (rec_out) {
    t2 = now();
    apf::Field* rec = spr::recoverField(grad);
    t3 = now();
    for (size_t i = 0; i < r->ents[0].size(); ++i) {
      apf::Vector3 g;
      apf::getVector(rec, r->ents[0][i], 0, g);
      for (int k = 0; k < 3; ++k) rec_out[3 * i + k] = g[k];
    }
    apf::destroyField(rec);
  }
  double t4 = now(), t5 = t4;
  if (size_out) {
    apf::Field* size = mode == 0 ? spr::getSPRSizeField(grad, adapt_ratio, the_pcu())
                                 : spr::getTargetSPRSizeField(grad, (size_t)target, the_pcu(), alpha, beta);
    t5 = now();
    for (size_t i = 0; i < r->ents[0].size(); ++i) size_out[i] = apf::getScalar(size, r->ents[0][i], 0);
    apf::destroyField(size);
  }
  apf::destroyField(grad);
  apf::destroyField(uf);
  if (seconds) {
    seconds[0] = t1 - t0;
    seconds[1] = t3 - t2;
    seconds[2] = t5 - t4;
  }
  return 0;
}

// ma::configure(m, size) (isotropic, ma/maInput.cc) on the vertex sizes, then
// mark_with; seconds[0] configure, [1..3] as mark_with
int refd_mark_iso(void* h, const double* size, double* lengths, int* flags, long* n_split, long* n_collapse,
                  double* quality, double* seconds) {
  RefMesh* r = (RefMesh*)h;
  apf::Field* sf = make_vertex_field(r, "refd_size", apf::SCALAR, size);
  double t0 = now();
  const ma::Input* in = ma::configure(r->m, sf);
  double t1 = now();
  int rc = mark_with(r, in, lengths, flags, n_split, n_collapse, quality, seconds ? seconds + 1 : nullptr);
  if (seconds) seconds[0] = t1 - t0;
  apf::destroyField(sf);
  return rc;
}

// ma::configure(m, sizes, frames, 0, log) (AnisoSizeField, or
// LogAnisoSizeField when log != 0) then mark_with.  sizes n_verts x 3,
// frames n_verts x 9 row-major.
int refd_mark_aniso(void* h, const double* sizes, const double* frames, int log, double* lengths, int* flags,
                    long* n_split, long* n_collapse, double* quality) {
  RefMesh* r = (RefMesh*)h;
  apf::Field* sz = make_vertex_field(r, "refd_sizes", apf::VECTOR, sizes);
  apf::Field* fr = make_vertex_field(r, "refd_frames", apf::MATRIX, frames);
  const ma::Input* in = ma::configure(r->m, sz, fr, nullptr, log != 0);
  int rc = mark_with(r, in, lengths, flags, n_split, n_collapse, quality, nullptr);
  if (log) {  // an AnisoSizeField destroys the sizes and frames fields it was given
    apf::destroyField(fr);
    apf::destroyField(sz);
  }
  return rc;
}

// The timed estimate-and-mark pass on field u: getGradIPField ->
// getSPRSizeField -> configure(m, size) -> markEdgesToCollapse ->
// markEdgesToSplit.  seconds[0..3]: gradient, size field, configure, marks.
int refd_pass(void* h, const double* u, double adapt_ratio, double* size_out, int* flags, long* n_split,
              long* n_collapse, double* seconds) {
  RefMesh* r = (RefMesh*)h;
  apf::Field* uf = make_vertex_field(r, "refd_u", apf::SCALAR, u);
  double t0 = now();
  apf::Field* grad = spr::getGradIPField(uf, "grad", 1);
  double t1 = now();
  apf::Field* size = spr::getSPRSizeField(grad, adapt_ratio, the_pcu());
  double t2 = now();
  const ma::Input* cin = ma::configure(r->m, size);
  double t3 = now();
  ma::Input* in = ma::makeAdvanced(cin);
  ma::Adapt* a = new ma::Adapt(in);
  const long nc = ma::markEdgesToCollapse(a);
  const long ns = ma::markEdgesToSplit(a);
  double t4 = now();
  if (size_out)
    for (size_t i = 0; i < r->ents[0].size(); ++i) size_out[i] = apf::getScalar(size, r->ents[0][i], 0);
  if (flags)
    for (size_t i = 0; i < r->ents[1].size(); ++i) flags[i] = ma::getFlags(a, r->ents[1][i]);
  if (n_split) *n_split = ns;
  if (n_collapse) *n_collapse = nc;
  if (seconds) {
    seconds[0] = t1 - t0;
    seconds[1] = t2 - t1;
    seconds[2] = t3 - t2;
    seconds[3] = t4 - t3;
  }
  delete a;
  if (in->ownsSolutionTransfer) delete in->solutionTransfer;
  delete in->sizeField;
  delete in;
  apf::destroyField(size);
  apf::destroyField(grad);
  apf::destroyField(uf);
  return 0;
}

}  // extern "C"
