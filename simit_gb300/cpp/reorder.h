// Set reordering of the C++ facade: the reference's simit::reorder,
// reorderVertexSet, reorderEdgeSet and reorderEdgeSetByVertexOrdering
// (src/reorder.h:11-32, src/reorder.cpp:222-273) on facade Sets.
//
// An ordering maps old to new: ordering[i] is the new index of element i,
// and a field's values move with their element, new[ordering[i]] = old[i]
// (the reference's reorderFieldData, src/reorder.h:35-49).
//
// reorder() sorts the vertices along a Hilbert curve over the spatial field
// (sg_hilbert_order) and then the elements by their sorted endpoint tuples
// (sg_element_order), as simit::reorder does (src/reorder.cpp:252-267); the
// curve is this library's, not the reference's hilbert_c2i, so the
// permutation differs while the locality is the same.  Both orderings it
// returns map old to new.
//
// One difference from the reference: its reorderEdgeSet gathers the
// endpoints through the map (new[e] = old[ordering[e]], src/reorder.cpp:
// 222-238) but scatters the fields through it, which agree only when the
// ordering is its own inverse.  Here endpoints and fields both move old to
// new, so an element's fields stay with its endpoints for any ordering.
#pragma once
#include <cstring>
#include <string>
#include <vector>

namespace simit_gb300 {

namespace detail {

inline void check_ordering(const std::vector<int> &ord, int size, const char *what) {
  if ((int)ord.size() != size)
    throw SimitException(std::string(what) + ": the ordering has " + std::to_string(ord.size()) +
                         " entries, the set " + std::to_string(size));
  std::vector<char> seen(size, 0);
  for (int i = 0; i < size; ++i) {
    const int k = ord[i];
    if (k < 0 || k >= size || seen[k])
      throw SimitException(std::string(what) + ": the ordering is not a permutation (entry " +
                           std::to_string(i) + " = " + std::to_string(k) + ")");
    seen[k] = 1;
  }
}

// new[ord[i]] = old[i] for every field, element by element.
inline void move_fields(Set &s, const std::vector<int> &ord) {
  for (FieldData &f : s.getFields()) {
    const size_t eb = (size_t)f.comps * f.elem_size();
    std::vector<unsigned char> out(f.data.size());
    for (size_t i = 0; i < ord.size(); ++i)
      std::memcpy(out.data() + (size_t)ord[i] * eb, f.data.data() + i * eb, eb);
    f.data.swap(out);
  }
}

}  // namespace detail

// Endpoints relabelled: each endpoint v becomes vertexOrdering[v].
inline void reorderEdgeSetByVertexOrdering(Set &edgeSet, const std::vector<int> &vertexOrdering) {
  int32_t *ep = edgeSet.getEndpointsPtr();
  const size_t m = (size_t)edgeSet.getSize() * edgeSet.getCardinality();
  for (size_t k = 0; k < m; ++k) {
    if (ep[k] < 0 || ep[k] >= (int)vertexOrdering.size())
      throw SimitException("reorderEdgeSetByVertexOrdering: endpoint " + std::to_string(ep[k]) +
                           " outside the ordering");
    ep[k] = vertexOrdering[ep[k]];
  }
}

// The vertex set's fields moved to their new indices and the edge set's
// endpoints relabelled.
inline void reorderVertexSet(Set &edgeSet, Set &vertexSet, std::vector<int> &vertexOrdering) {
  detail::check_ordering(vertexOrdering, vertexSet.getSize(), "reorderVertexSet");
  reorderEdgeSetByVertexOrdering(edgeSet, vertexOrdering);
  detail::move_fields(vertexSet, vertexOrdering);
}

// The edge set's elements (endpoints and fields) moved to their new indices.
inline void reorderEdgeSet(Set &edgeSet, const std::vector<int> &edgeOrdering) {
  detail::check_ordering(edgeOrdering, edgeSet.getSize(), "reorderEdgeSet");
  const int card = edgeSet.getCardinality();
  int32_t *ep = edgeSet.getEndpointsPtr();
  std::vector<int32_t> out((size_t)edgeSet.getSize() * card);
  for (size_t i = 0; i < edgeOrdering.size(); ++i)
    std::memcpy(out.data() + (size_t)edgeOrdering[i] * card, ep + i * card,
                card * sizeof(int32_t));
  if (!out.empty()) std::memcpy(ep, out.data(), out.size() * sizeof(int32_t));
  detail::move_fields(edgeSet, edgeOrdering);
}

// Vertices along the Hilbert curve of the spatial field (3 components,
// double or float), then elements by sorted endpoint tuples; the orderings
// applied are returned, old to new.
inline void reorder(Set &edgeSet, Set &vertexSet, std::vector<int> &edgeOrdering,
                    std::vector<int> &vertexOrdering, int bits = 10) {
  if (!vertexSet.hasSpatialField())
    throw SimitException("reorder: the vertex set needs a spatial field (setSpatialField)");
  FieldData *xf = vertexSet.field(vertexSet.getSpatialFieldName());
  if (!xf || xf->comps != 3 || (xf->type != FieldType::F64 && xf->type != FieldType::F32))
    throw SimitException("reorder: the spatial field must hold 3 floating-point components");
  const int n = vertexSet.getSize();
  std::vector<double> xyz((size_t)n * 3);
  for (size_t k = 0; k < xyz.size(); ++k)
    xyz[k] = xf->type == FieldType::F64 ? reinterpret_cast<const double *>(xf->data.data())[k]
                                        : reinterpret_cast<const float *>(xf->data.data())[k];
  vertexOrdering.assign(n, 0);
  check(sg_hilbert_order(n, xyz.data(), bits, vertexOrdering.data()), "reorder");
  reorderVertexSet(edgeSet, vertexSet, vertexOrdering);
  const int nE = edgeSet.getSize();
  std::vector<int> newToOld(nE);
  check(sg_element_order(nE, edgeSet.getCardinality(), edgeSet.getEndpointsPtr(),
                         newToOld.data()),
        "reorder");
  edgeOrdering.assign(nE, 0);
  for (int k = 0; k < nE; ++k) edgeOrdering[newToOld[k]] = k;
  reorderEdgeSet(edgeSet, edgeOrdering);
}

inline void reorder(Set &edgeSet, Set &vertexSet) {
  std::vector<int> e, v;
  reorder(edgeSet, vertexSet, e, v);
}

}  // namespace simit_gb300
