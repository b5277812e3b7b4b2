// Locality renumbering of a flattened mesh: the flat-array counterpart of
// apf::reorderMdsMesh (mds/apfMDS.cc:957 -> mds_reorder, mds/mds_order.c:409).
//
// The reference numbers the vertices breadth-first from a seed
// (mds_number_verts_bfs, mds/mds_order.c:127-141): the seed is the first
// vertex on the lowest-dimension model entity, a vertex's neighbours are
// visited in the order of its upward edge list, and vertices left over
// (other components) start new searches in index order.  Every other entity
// is then numbered in the order the renumbered vertices first reach it
// (number_other_ents, :158-176).  A flattened view carries no geometric
// model, so the seed here is the first vertex of the smallest degree (a
// domain corner on structured meshes, where the reference's seed is a model
// vertex); neighbours are visited in descending edge id (the upward list of
// MDS holds the newest edge first), elements in the order of each vertex's
// element adjacency (the view's getAdjacent CSR when it has one, else
// ascending) and edges in descending id.
//
// Renumbered meshes keep every element's and edge's own vertex order, so
// orientation and downward order are unchanged.  Host code only.
#include <algorithm>
#include <vector>

#include "spr_gb300.h"

extern "C" int sprg_locality_order(const sprg_mesh_view* mv, int32_t* vert_new, int32_t* elem_new,
                                   int32_t* edge_new) {
  if (!mv || !vert_new || !elem_new || !edge_new) return SPRG_EINVAL;
  if ((mv->dim != 2 && mv->dim != 3) || mv->n_verts <= 0 || mv->n_elems < 0 || mv->n_edges < 0) return SPRG_EINVAL;
  if (mv->n_verts > INT32_MAX || mv->n_elems > INT32_MAX || mv->n_edges > INT32_MAX / 2) return SPRG_EINVAL;
  if (!mv->elem_verts || (mv->n_edges && !mv->edge_verts)) return SPRG_EINVAL;
  if ((mv->vert_elem_offsets == nullptr) != (mv->vert_elems == nullptr)) return SPRG_EINVAL;
  const int64_t V = mv->n_verts, T = mv->n_elems, E = mv->n_edges;
  const int nn = mv->dim + 1;
  for (int64_t i = 0; i < T * nn; ++i)
    if (mv->elem_verts[i] < 0 || mv->elem_verts[i] >= V) return SPRG_EINVAL;
  for (int64_t i = 0; i < 2 * E; ++i)
    if (mv->edge_verts[i] < 0 || mv->edge_verts[i] >= V) return SPRG_EINVAL;

  // vertex -> edge adjacency, each row in descending edge id
  std::vector<int64_t> eoff(V + 1, 0);
  for (int64_t e = 0; e < E; ++e) {
    ++eoff[mv->edge_verts[2 * e] + 1];
    ++eoff[mv->edge_verts[2 * e + 1] + 1];
  }
  for (int64_t v = 0; v < V; ++v) eoff[v + 1] += eoff[v];
  std::vector<int32_t> eadj(eoff[V]);
  {
    std::vector<int64_t> pos(eoff.begin(), eoff.end() - 1);
    for (int64_t e = E - 1; e >= 0; --e) {
      eadj[pos[mv->edge_verts[2 * e]]++] = (int32_t)e;
      eadj[pos[mv->edge_verts[2 * e + 1]]++] = (int32_t)e;
    }
  }
  // vertex -> element adjacency: the view's getAdjacent order, else ascending
  std::vector<int64_t> toff(V + 1, 0);
  std::vector<int32_t> tadj;
  if (mv->vert_elem_offsets) {
    if (mv->vert_elem_offsets[0] != 0 || mv->vert_elem_offsets[V] != T * nn) return SPRG_EINVAL;
    for (int64_t v = 0; v <= V; ++v) toff[v] = mv->vert_elem_offsets[v];
    for (int64_t v = 0; v < V; ++v)
      if (toff[v + 1] < toff[v]) return SPRG_EINVAL;
    tadj.assign(mv->vert_elems, mv->vert_elems + T * nn);
    for (int32_t t : tadj)
      if (t < 0 || t >= T) return SPRG_EINVAL;
  } else {
    for (int64_t i = 0; i < T * nn; ++i) ++toff[mv->elem_verts[i] + 1];
    for (int64_t v = 0; v < V; ++v) toff[v + 1] += toff[v];
    tadj.resize(T * nn);
    std::vector<int64_t> pos(toff.begin(), toff.end() - 1);
    for (int64_t t = 0; t < T; ++t)
      for (int k = 0; k < nn; ++k) tadj[pos[mv->elem_verts[t * nn + k]]++] = (int32_t)t;
  }

  // vertices: breadth-first from the seed, then from every vertex not reached
  std::fill(vert_new, vert_new + V, -1);
  std::vector<int32_t> order;
  order.reserve(V);
  int64_t seed = 0;
  for (int64_t v = 1; v < V; ++v)
    if (eoff[v + 1] - eoff[v] < eoff[seed + 1] - eoff[seed]) seed = v;
  auto search = [&](int64_t s) {
    if (vert_new[s] >= 0) return;
    size_t head = order.size();
    vert_new[s] = (int32_t)order.size();
    order.push_back((int32_t)s);
    while (head < order.size()) {
      const int32_t v = order[head++];
      for (int64_t j = eoff[v]; j < eoff[v + 1]; ++j) {
        const int32_t e = eadj[j];
        const int32_t w = mv->edge_verts[2 * e] == v ? mv->edge_verts[2 * e + 1] : mv->edge_verts[2 * e];
        if (vert_new[w] < 0) {
          vert_new[w] = (int32_t)order.size();
          order.push_back(w);
        }
      }
    }
  };
  search(seed);
  for (int64_t v = 0; v < V; ++v) search(v);

  // elements and edges in the order the renumbered vertices reach them
  std::fill(elem_new, elem_new + T, -1);
  std::fill(edge_new, edge_new + E, -1);
  int32_t nt = 0, ne = 0;
  for (int32_t v : order) {
    for (int64_t j = toff[v]; j < toff[v + 1]; ++j)
      if (elem_new[tadj[j]] < 0) elem_new[tadj[j]] = nt++;
    for (int64_t j = eoff[v]; j < eoff[v + 1]; ++j)
      if (edge_new[eadj[j]] < 0) edge_new[eadj[j]] = ne++;
  }
  // elements outside the adjacency (none in a valid view) keep their order at the end
  for (int64_t t = 0; t < T; ++t)
    if (elem_new[t] < 0) elem_new[t] = nt++;
  for (int64_t e = 0; e < E; ++e)
    if (edge_new[e] < 0) edge_new[e] = ne++;
  return SPRG_OK;
}
