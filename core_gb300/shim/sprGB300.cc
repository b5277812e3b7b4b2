// sprGB300.cc -- the reference-side drop-in of the GB300 estimate-and-mark
// pass (declarations and conventions in sprGB300.h).  Built inside a
// SCOREC/core tree against its apf, mds, spr and ma headers and linked with
// libsprgb300.so.
#include "sprGB300.h"

#include <apfMDS.h>
#include <apfShape.h>
#include <lionPrint.h>
#include <maSize.h>

#include <map>
#include <string>

namespace gb300 {
namespace {

struct Entry {
  Flat flat;
  sprg_ctx* ctx = nullptr;
  int precision = SPRG_FP64;
  // the size field(s) recorded by ma::gb300::configure for the marks
  apf::Field* size = nullptr;
  apf::Field* sizes = nullptr;
  apf::Field* frames = nullptr;
  bool log = false;
};

std::map<apf::Mesh*, Entry>& registry() {
  static std::map<apf::Mesh*, Entry> r;
  return r;
}

void check(sprg_ctx* c, int rc) {
  if (rc) apf::fail(c ? sprg_last_error(c) : "GB300 estimate-and-mark call failed");
}

apf::Mesh2* mesh2(apf::Mesh* m) {
  apf::Mesh2* m2 = dynamic_cast<apf::Mesh2*>(m);
  if (!m2) apf::fail("GB300 pass: the field's mesh is not an apf::Mesh2");
  return m2;
}

Entry& entry(apf::Mesh2* m) {
  Entry& e = registry()[m];
  if (!e.ctx) {
    e.flat = flatten(m);
    const sprg_mesh_view v = e.flat.view();
    sprg_ctx* c = nullptr;
    if (sprg_create(&v, 0, &c)) apf::fail("GB300 pass: sprg_create refused the mesh");
    e.ctx = c;
    if (e.precision != SPRG_FP64) check(c, sprg_set_precision(c, e.precision));
  }
  return e;
}

// a field's values at the nodes of one dimension, in MDS index order
std::vector<double> values_on(apf::Mesh2* m, apf::Field* f, int dim) {
  const int nc = apf::countComponents(f);
  std::vector<double> out((size_t)m->count(dim) * nc);
  apf::MeshIterator* it = m->begin(dim);
  apf::MeshEntity* e;
  while ((e = m->iterate(it))) apf::getComponents(f, e, 0, &out[(size_t)nc * apf::getMdsIndex(m, e)]);
  m->end(it);
  return out;
}

void set_values_on(apf::Mesh2* m, apf::Field* f, int dim, const std::vector<double>& vals) {
  const int nc = apf::countComponents(f);
  apf::MeshIterator* it = m->begin(dim);
  apf::MeshEntity* e;
  while ((e = m->iterate(it))) apf::setComponents(f, e, 0, &vals[(size_t)nc * apf::getMdsIndex(m, e)]);
  m->end(it);
}

}  // namespace

sprg_mesh_view Flat::view() const {
  sprg_mesh_view v;
  v.dim = dim;
  v.n_verts = (int64_t)(xyz.size() / 3);
  v.n_elems = (int64_t)(ev.size() / (dim + 1));
  v.n_edges = (int64_t)(ed.size() / 2);
  v.coords = xyz.data();
  v.elem_verts = ev.data();
  v.edge_verts = ed.data();
  v.vert_elem_offsets = off.data();
  v.vert_elems = adj.data();
  return v;
}

Flat flatten(apf::Mesh2* m) {
  Flat f;
  f.dim = m->getDimension();
  const size_t V = m->count(0), T = m->count(f.dim), E = m->count(1);
  const int nn = f.dim + 1;
  f.xyz.resize(3 * V);
  f.ev.resize(nn * T);
  f.ed.resize(2 * E);
  std::vector<std::vector<int32_t>> up(V);
  apf::MeshIterator* it = m->begin(0);
  apf::MeshEntity* e;
  while ((e = m->iterate(it))) {
    const int i = apf::getMdsIndex(m, e);
    apf::Vector3 p;
    m->getPoint(e, 0, p);
    for (int k = 0; k < 3; ++k) f.xyz[3 * (size_t)i + k] = p[k];
    apf::Adjacent a;
    m->getAdjacent(e, f.dim, a);  // the reference's averaging order
    for (size_t j = 0; j < a.getSize(); ++j) up[i].push_back(apf::getMdsIndex(m, a[j]));
  }
  m->end(it);
  f.off.resize(V + 1);
  f.off[0] = 0;
  for (size_t i = 0; i < V; ++i) {
    f.off[i + 1] = f.off[i] + (int32_t)up[i].size();
    f.adj.insert(f.adj.end(), up[i].begin(), up[i].end());
  }
  apf::Downward dv;
  it = m->begin(f.dim);
  while ((e = m->iterate(it))) {
    const size_t i = apf::getMdsIndex(m, e);
    m->getDownward(e, 0, dv);
    for (int k = 0; k < nn; ++k) f.ev[nn * i + k] = apf::getMdsIndex(m, dv[k]);
  }
  m->end(it);
  it = m->begin(1);
  while ((e = m->iterate(it))) {
    const size_t i = apf::getMdsIndex(m, e);
    m->getDownward(e, 0, dv);
    f.ed[2 * i] = apf::getMdsIndex(m, dv[0]);
    f.ed[2 * i + 1] = apf::getMdsIndex(m, dv[1]);
  }
  m->end(it);
  return f;
}

sprg_ctx* context(apf::Mesh2* m) { return entry(m).ctx; }

void setPrecision(apf::Mesh2* m, int precision) {
  Entry& e = registry()[m];
  e.precision = precision;
  if (e.ctx) check(e.ctx, sprg_set_precision(e.ctx, precision));
}

void invalidate(apf::Mesh2* m) {
  auto it = registry().find(m);
  if (it == registry().end()) return;
  if (it->second.ctx) sprg_destroy(it->second.ctx);
  it->second.ctx = nullptr;
  it->second.flat = Flat();
}

std::vector<int32_t> readEdgeFlags(ma::Adapt* a) {
  apf::Mesh2* m = a->mesh;
  std::vector<int32_t> flags(m->count(1));
  apf::MeshIterator* it = m->begin(1);
  apf::MeshEntity* e;
  while ((e = m->iterate(it))) flags[apf::getMdsIndex(m, e)] = ma::getFlags(a, e);
  m->end(it);
  return flags;
}

void writeEdgeFlags(ma::Adapt* a, const std::vector<int32_t>& flags) {
  apf::Mesh2* m = a->mesh;
  apf::MeshIterator* it = m->begin(1);
  apf::MeshEntity* e;
  while ((e = m->iterate(it))) ma::setFlags(a, e, flags[apf::getMdsIndex(m, e)]);
  m->end(it);
}

// the recorded size field's inputs for the C ABI (kind, sizes), or fail
static int size_kind(Entry& en, apf::Mesh2* m, std::vector<double>& s1, std::vector<double>& s3,
                     std::vector<double>& f9) {
  if (en.size) {
    s1 = values_on(m, en.size, 0);
    return SPRG_SIZE_ISO;
  }
  if (en.sizes && en.frames) {
    s3 = values_on(m, en.sizes, 0);
    f9 = values_on(m, en.frames, 0);
    return en.log ? SPRG_SIZE_LOG_ANISO : SPRG_SIZE_ANISO;
  }
  apf::fail("GB300 pass: no size field recorded for this mesh (use ma::gb300::configure)");
  return -1;
}

}  // namespace gb300

namespace spr {
namespace gb300 {

apf::Field* getGradIPField(apf::Field* f, const char* name, int order) {
  apf::Mesh2* m = ::gb300::mesh2(apf::getMesh(f));
  const int vt = apf::getValueType(f);
  if (vt != apf::SCALAR && vt != apf::VECTOR) apf::fail("GB300 getGradIPField: SCALAR or VECTOR fields");
  ::gb300::Entry& en = ::gb300::entry(m);
  const int ncin = apf::countComponents(f);
  std::vector<double> u = ::gb300::values_on(m, f, 0);
  std::vector<double> ip((size_t)m->count(m->getDimension()) * 3 * ncin);
  ::gb300::check(en.ctx, sprg_get_grad_ip_field(en.ctx, u.data(), ncin, order, ip.data()));
  apf::Field* out = apf::createIPField(m, name, vt + 1, order);
  ::gb300::set_values_on(m, out, m->getDimension(), ip);
  return out;
}

apf::Field* recoverField(apf::Field* ip_field) {
  apf::Mesh2* m = ::gb300::mesh2(apf::getMesh(ip_field));
  ::gb300::Entry& en = ::gb300::entry(m);
  const int nc = apf::countComponents(ip_field);
  std::vector<double> ip = ::gb300::values_on(m, ip_field, m->getDimension());
  std::vector<double> rec((size_t)m->count(0) * nc);
  ::gb300::check(en.ctx, sprg_recover_field(en.ctx, ip.data(), nc, rec.data()));
  std::string name = "spr_";
  name += apf::getName(ip_field);
  apf::Field* out = apf::createLagrangeField(m, name.c_str(), apf::getValueType(ip_field), 1);
  ::gb300::set_values_on(m, out, 0, rec);
  return out;
}

static apf::Field* size_field(apf::Field* eps, int mode, double adapt_ratio, size_t target, double alpha, double beta,
                              pcu::PCU* PCUObj) {
  apf::Mesh2* m = ::gb300::mesh2(apf::getMesh(eps));
  ::gb300::Entry& en = ::gb300::entry(m);
  const double t0 = pcu::Time();
  const int nc = apf::countComponents(eps);
  std::vector<double> ip = ::gb300::values_on(m, eps, m->getDimension());
  std::vector<double> size(m->count(0));
  sprg_size_info info;
  if (mode == 0)
    ::gb300::check(en.ctx, sprg_get_spr_size_field(en.ctx, ip.data(), nc, adapt_ratio, size.data(), &info));
  else
    ::gb300::check(en.ctx, sprg_get_target_spr_size_field(en.ctx, ip.data(), nc, target, alpha, beta, size.data(),
                                                          &info));
  apf::Field* out = apf::createLagrangeField(m, "size", apf::SCALAR, 1);
  ::gb300::set_values_on(m, out, 0, size);
  if (!PCUObj->Self())
    lion_eprint(1, "SPR%s (GB300): error estimated in %f seconds\n", mode ? " (target)" : "", pcu::Time() - t0);
  return out;
}

apf::Field* getSPRSizeField(apf::Field* eps, double adapt_ratio, pcu::PCU* PCUObj) {
  return size_field(eps, 0, adapt_ratio, 0, 0, 0, PCUObj);
}

apf::Field* getTargetSPRSizeField(apf::Field* eps, size_t target, pcu::PCU* PCUObj, double alpha, double beta) {
  if (!(target > 0) || !(alpha < beta)) apf::fail("GB300 getTargetSPRSizeField: target > 0 and alpha < beta");
  return size_field(eps, 1, 0, target, alpha, beta, PCUObj);
}

}  // namespace gb300
}  // namespace spr

namespace ma {
namespace gb300 {

const Input* configure(Mesh* m, apf::Field* size, SolutionTransfer* s) {
  ::gb300::Entry& en = ::gb300::registry()[m];
  en.size = size;
  en.sizes = en.frames = nullptr;
  return ma::configure(m, size, s);
}

const Input* configure(Mesh* m, apf::Field* sizes, apf::Field* frames, SolutionTransfer* s, bool logInterpolation) {
  ::gb300::Entry& en = ::gb300::registry()[m];
  en.size = nullptr;
  en.sizes = sizes;
  en.frames = frames;
  en.log = logInterpolation;
  return ma::configure(m, sizes, frames, s, logInterpolation);
}

// lengths of every edge under the recorded size field, resident on the device
static void measure(::gb300::Entry& en, Mesh* m) {
  std::vector<double> s1, s3, f9;
  const int kind = ::gb300::size_kind(en, m, s1, s3, f9);
  if (kind == SPRG_SIZE_ISO) ::gb300::check(en.ctx, sprg_measure_edges(en.ctx, s1.data(), nullptr));
  else if (kind == SPRG_SIZE_ANISO)
    ::gb300::check(en.ctx, sprg_measure_edges_aniso(en.ctx, s3.data(), f9.data(), nullptr));
  else ::gb300::check(en.ctx, sprg_measure_edges_log_aniso(en.ctx, s3.data(), f9.data(), nullptr));
}

static long mark(Adapt* a, int which) {
  ::gb300::Entry& en = ::gb300::entry(a->mesh);
  measure(en, a->mesh);
  std::vector<int32_t> flags = ::gb300::readEdgeFlags(a);
  long n = 0;
  ::gb300::check(en.ctx, sprg_mark_edges(en.ctx, which, flags.data(), &n));
  ::gb300::writeEdgeFlags(a, flags);
  return a->mesh->getPCU()->Add<long>(n);
}

long markEdgesToSplit(Adapt* a) { return mark(a, SPRG_MARK_SPLIT); }
long markEdgesToCollapse(Adapt* a) { return mark(a, SPRG_MARK_COLLAPSE); }

double getMaximumEdgeLength(Mesh* m, SizeField* sf) {
  ::gb300::Entry& en = ::gb300::entry(m);
  double L = 0;
  if (!sf) {
    ::gb300::check(en.ctx, sprg_get_maximum_edge_length(en.ctx, SPRG_SIZE_IDENTITY, nullptr, nullptr, nullptr, &L));
  } else {
    std::vector<double> s1, s3, f9;
    const int kind = ::gb300::size_kind(en, m, s1, s3, f9);
    ::gb300::check(en.ctx, sprg_get_maximum_edge_length(en.ctx, kind, s1.empty() ? nullptr : s1.data(),
                                                        s3.empty() ? nullptr : s3.data(),
                                                        f9.empty() ? nullptr : f9.data(), &L));
  }
  return m->getPCU()->Max<double>(L);
}

double getMinQuality(Adapt* a) {
  ::gb300::Entry& en = ::gb300::entry(a->mesh);
  std::vector<double> s1, s3, f9;
  const int kind = ::gb300::size_kind(en, a->mesh, s1, s3, f9);
  std::vector<double> q(a->mesh->count(a->mesh->getDimension()));
  if (kind == SPRG_SIZE_LOG_ANISO)
    ::gb300::check(en.ctx, sprg_measure_quality_log_aniso(en.ctx, s3.data(), f9.data(), q.data()));
  else
    ::gb300::check(en.ctx, sprg_measure_quality(en.ctx, s1.empty() ? nullptr : s1.data(),
                                                s3.empty() ? nullptr : s3.data(),
                                                f9.empty() ? nullptr : f9.data(), q.data()));
  double mq = 1;
  ::gb300::check(en.ctx, sprg_get_min_quality(en.ctx, &mq));
  return a->mesh->getPCU()->Min<double>(mq);
}

}  // namespace gb300
}  // namespace ma
