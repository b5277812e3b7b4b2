/*
 * sprGB300.h -- the reference-side drop-in of the GB300 estimate-and-mark
 * pass: what a SCOREC/core maintainer adds to spr/ and ma/ so that callers
 * keep the spr::/ma:: signatures and the work runs through the C ABI of
 * include/spr_gb300.h.
 *
 * Every function below has the signature of the reference call it replaces
 * (named beside it), in a nested `gb300` namespace: a caller switches by
 * writing spr::gb300::getSPRSizeField(...) for spr::getSPRSizeField(...).
 * The device side keeps one context per apf::Mesh2 (the flattened mesh, its
 * per-mesh caches), created on first use; after the mesh changes (refine,
 * coarsen, snap, or new coordinates) the caller calls gb300::invalidate(m)
 * before the next call.  Fields come back as the reference creates them
 * (names, shapes, value types, owned by the mesh).  A nonzero status of the
 * C ABI becomes apf::fail, as the reference aborts.
 *
 * Isotropic and anisotropic size fields for the marks: the configure
 * drop-ins below build the stock ma::Input (so every other MA operator is
 * unchanged) and record the size field(s) for the mesh; markEdgesToSplit /
 * markEdgesToCollapse then measure those sizes on the GPU and write the
 * ma_flags words exactly as ma::markEntities does.
 */
#ifndef SPR_GB300_SHIM_H
#define SPR_GB300_SHIM_H

#include <apf.h>
#include <apfMesh2.h>
#include <PCU.h>
#include <maAdapt.h>
#include <maInput.h>

#include <stdint.h>
#include <vector>

#include "spr_gb300.h"

namespace gb300 {

/* A flattened mesh in MDS index order: exactly what sprg_mesh_view carries
   (coordinates, element and edge vertices, the vertex-to-element adjacency
   in getAdjacent(v, dim) order). */
struct Flat {
  int dim = 0;
  std::vector<double> xyz;
  std::vector<int32_t> ev, ed, off, adj;
  sprg_mesh_view view() const;
};

/* The MDS-to-device flattener's host half: one pass over the mesh's
   entities (apf::getMdsIndex numbering). */
Flat flatten(apf::Mesh2* m);

/* The device context of a mesh (created on first use: device 0, the
   precision set by setPrecision, SPRG_FP64 by default). */
sprg_ctx* context(apf::Mesh2* m);
/* SPRG_FP64, SPRG_FP32 or SPRG_LEARNED for the mesh's context. */
void setPrecision(apf::Mesh2* m, int precision);
/* Drop the mesh's context after it changed; the next call re-flattens. */
void invalidate(apf::Mesh2* m);

/* ma_flags words of every edge (MDS order) and their write-back. */
std::vector<int32_t> readEdgeFlags(ma::Adapt* a);
void writeEdgeFlags(ma::Adapt* a, const std::vector<int32_t>& flags);

}  // namespace gb300

namespace spr {
namespace gb300 {

/* spr::getGradIPField (spr/spr.h:33, spr/sprGetGradIPField.cc:15) */
apf::Field* getGradIPField(apf::Field* f, const char* name, int order);
/* spr::recoverField (spr/spr.h:39, spr/sprRecoverField.cc:419) */
apf::Field* recoverField(apf::Field* ip_field);
/* spr::getSPRSizeField (spr/spr.h:47, spr/sprEstimateError.cc:311) */
apf::Field* getSPRSizeField(apf::Field* eps, double adapt_ratio, pcu::PCU* PCUObj);
/* spr::getTargetSPRSizeField (spr/spr.h:56, spr/sprEstimateTargetError.cc:241) */
apf::Field* getTargetSPRSizeField(apf::Field* eps, size_t target, pcu::PCU* PCUObj, double alpha = 0.25,
                                  double beta = 2.0);

}  // namespace gb300
}  // namespace spr

namespace ma {
namespace gb300 {

/* ma::configure(m, size, s) (ma/maInput.h:203): the stock Input, and `size`
   recorded as the mesh's isotropic size field for the marks below */
const Input* configure(Mesh* m, apf::Field* size, SolutionTransfer* s = 0);
/* ma::configure(m, sizes, frames, s, logInterpolation) (ma/maInput.h:193) */
const Input* configure(Mesh* m, apf::Field* sizes, apf::Field* frames, SolutionTransfer* s = 0,
                       bool logInterpolation = true);
/* ma::markEdgesToSplit (ma/maRefine.h:52, ma/maRefine.cc:395) */
long markEdgesToSplit(Adapt* a);
/* ma::markEdgesToCollapse (ma/maCoarsen.cc:287) */
long markEdgesToCollapse(Adapt* a);
/* ma::getMaximumEdgeLength (ma/maSize.h:116): sf = 0 is the identity size
   field, otherwise the recorded size field of the mesh */
double getMaximumEdgeLength(Mesh* m, SizeField* sf = 0);
/* ma::getMinQuality (ma/maShape.cc:151) under the recorded size field */
double getMinQuality(Adapt* a);

}  // namespace gb300
}  // namespace ma

#endif
