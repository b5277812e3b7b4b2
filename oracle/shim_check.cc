// C entry points that exercise the reference-side shim (core_gb300/shim)
// on real apf::Mesh2 meshes of the reference -- TEST INFRASTRUCTURE ONLY.
//
// Built by `make -C oracle shim REF=<tree>` against the reference compiled
// from source (oracle/_ref/libspr_ref.a) and the product library.  The shim's
// device calls need a GPU, which the hosts with the reference tree lack, so
// these checks cover its host half: the flattener's arrays against the
// reference's own numbering, and the ma_flags round trip through
// gb300::readEdgeFlags / sprg_apply_marks / gb300::writeEdgeFlags against
// the stock ma::markEdgesToCollapse / ma::markEdgesToSplit.
#include <apfBox.h>
#include <apfMDS.h>
#include <gmi_mesh.h>
#include <gmi_null.h>
#include <lionPrint.h>
#include <ma.h>
#include <maRefine.h>
#include <maSize.h>

#include <cstring>

#include "sprGB300.h"

namespace ma {
long markEdgesToCollapse(Adapt* a);  // ma/maCoarsen.cc:287 (no header declaration)
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

void copy_flat(const gb300::Flat& f, double* coords, int* ev, int* ed, int* off, int* adj) {
  std::memcpy(coords, f.xyz.data(), sizeof(double) * f.xyz.size());
  std::memcpy(ev, f.ev.data(), sizeof(int) * f.ev.size());
  std::memcpy(ed, f.ed.data(), sizeof(int) * f.ed.size());
  std::memcpy(off, f.off.data(), sizeof(int) * f.off.size());
  std::memcpy(adj, f.adj.data(), sizeof(int) * f.adj.size());
}

void destroy(apf::Mesh2* m) {
  m->destroyNative();
  apf::destroyMesh(m);
}

}  // namespace

extern "C" {

// gb300::flatten of apf::makeMdsBox(nx, ny, nz, 1, 1, 1 (0 when nz = 0), true)
void shimchk_flatten_box(int nx, int ny, int nz, double* coords, int* ev, int* ed, int* off, int* adj) {
  apf::Mesh2* m = apf::makeMdsBox(nx, ny, nz, 1, 1, nz ? 1 : 0, true, the_pcu());
  copy_flat(gb300::flatten(m), coords, ev, ed, off, adj);
  destroy(m);
}

// counts and gb300::flatten of a .smb mesh on the null model (name without
// the part number, as apf::loadMdsMesh takes it); arrays may be NULL to ask
// for the counts (dim, V, T, E, adjacency length) only
void shimchk_flatten_smb(const char* smb, long* counts, double* coords, int* ev, int* ed, int* off, int* adj) {
  gmi_model* g = (the_pcu(), gmi_load(".null"));
  apf::Mesh2* m = apf::loadMdsMesh(g, smb, the_pcu());
  gb300::Flat f = gb300::flatten(m);
  counts[0] = f.dim;
  counts[1] = (long)(f.xyz.size() / 3);
  counts[2] = (long)(f.ev.size() / (f.dim + 1));
  counts[3] = (long)(f.ed.size() / 2);
  counts[4] = (long)f.adj.size();
  if (coords) copy_flat(f, coords, ev, ed, off, adj);
  destroy(m);
}

// ma_flags after the collapse and split passes on a box with the given
// coordinates and vertex sizes, twice: flags_ref from the stock
// ma::markEdgesToCollapse / ma::markEdgesToSplit, flags_shim from the shim's
// flag I/O around sprg_apply_marks with the bitmaps of the stock size
// field's lengths.  prior (may be NULL): ma_flags words set on every edge
// before either pass.  counts: split / collapse of each.
int shimchk_marks(int nx, int ny, int nz, const double* coords, const double* size, const int* prior,
                  int* flags_ref, int* flags_shim, long* counts) {
  apf::Mesh2* m = apf::makeMdsBox(nx, ny, nz, 1, 1, nz ? 1 : 0, true, the_pcu());
  const size_t V = m->count(0), E = m->count(1);
  apf::MeshIterator* it = m->begin(0);
  apf::MeshEntity* e;
  while ((e = m->iterate(it))) {
    const int i = apf::getMdsIndex(m, e);
    m->setPoint(e, 0, apf::Vector3(coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]));
  }
  m->end(it);
  apf::Field* sf = apf::createFieldOn(m, "chk_size", apf::SCALAR);
  it = m->begin(0);
  while ((e = m->iterate(it))) apf::setScalar(sf, e, 0, size[apf::getMdsIndex(m, e)]);
  m->end(it);
  for (int pass = 0; pass < 2; ++pass) {
    ma::Input* in = ma::makeAdvanced(ma::configure(m, sf));
    ma::Adapt* a = new ma::Adapt(in);
    if (prior) {
      std::vector<int32_t> p(prior, prior + E);
      gb300::writeEdgeFlags(a, p);
    }
    long ns = 0, nc = 0;
    if (pass == 0) {
      nc = ma::markEdgesToCollapse(a);
      ns = ma::markEdgesToSplit(a);
    } else {
      std::vector<uint32_t> split((E + 31) / 32, 0u), collapse((E + 31) / 32, 0u);
      it = m->begin(1);
      while ((e = m->iterate(it))) {
        const size_t i = apf::getMdsIndex(m, e);
        const double L = in->sizeField->measure(e);
        if (L > ma::MAXLENGTH) split[i >> 5] |= 1u << (i & 31);
        if (L < ma::MINLENGTH) collapse[i >> 5] |= 1u << (i & 31);
      }
      m->end(it);
      std::vector<int32_t> flags = gb300::readEdgeFlags(a);
      const int rc = sprg_apply_marks((int64_t)E, split.data(), collapse.data(), flags.data(), &ns, &nc);
      if (rc) return rc;
      gb300::writeEdgeFlags(a, flags);
    }
    std::vector<int32_t> got = gb300::readEdgeFlags(a);
    std::memcpy(pass == 0 ? flags_ref : flags_shim, got.data(), sizeof(int) * E);
    counts[2 * pass] = ns;
    counts[2 * pass + 1] = nc;
    delete a;
    if (in->ownsSolutionTransfer) delete in->solutionTransfer;
    delete in->sizeField;
    delete in;
  }
  (void)V;
  apf::destroyField(sf);
  destroy(m);
  return 0;
}

}  // extern "C"
