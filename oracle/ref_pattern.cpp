// Test infrastructure only: a thin C driver around the reference's OWN pattern
// builder, compiled from the reference sources where they lie (see
// oracle/build_ref.sh).  It is never linked into the product library; tests use
// it to pin the oracle restatement (oracle/sg_oracle.cpp) bit-exactly.
//
// What it calls, and where the reference does the same:
//   * simit::Set with `card` endpoint sets, filled with Set::add
//       (src/graph.h:91-749, src/graph.cpp:18-29)
//   * the assembly path expression  ∃e∈E.(v-e ∧ e-u)
//       built exactly as src/path_expression_analysis.cpp:84-91 builds it
//   * pe::PathIndexBuilder::buildSegmented(pexpr, 0)
//       (src/path_indices.cpp:148-531), giving coords (n+1) and sinks (nnz)
//   * the runtime's own `loc` slot search (src/runtime.cpp:19-23), called per
//     element and endpoint pair in gatherVVLocs order (src/inline.cpp:544-552).
#include <cstdint>
#include <cstring>
#include <vector>

#include "graph.h"
#include "path_expressions.h"
#include "path_indices.h"

using namespace simit;
using namespace simit::pe;

extern "C" int loc(int v0, int v1, int *neighbors_start, int *neighbors);

namespace {

template <typename... Sets>
int64_t build_with(simit::Set &V, std::vector<ElementRef> &vrefs,
                   simit::Set &E, const int32_t *ep, int64_t nE, int card,
                   uint32_t *rowptr, uint32_t *colidx, int64_t cap) {
  (void)vrefs;
  PathIndexBuilder builder;
  builder.bind("V", &V);
  builder.bind("E", &E);
  Var v("v", pe::Set("V"));
  Var u("u", pe::Set("V"));
  Var e("e", pe::Set("E"));
  PathExpression ve = Link::make(v, e, Link::ve);
  PathExpression ev = Link::make(e, u, Link::ev);
  PathExpression vev = And::make({v, u}, {{QuantifiedVar::Exist, e}},
                                 ve(v, e), ev(e, u));
  PathIndex pidx = builder.buildSegmented(vev, 0);
  const int64_t n = (int64_t)pidx.numElements();
  int64_t k = 0;
  for (int64_t r = 0; r < n; ++r) {
    rowptr[r] = (uint32_t)k;
    for (unsigned c : pidx.neighbors((unsigned)r)) {
      if (k >= cap) return -1;
      colidx[k++] = c;
    }
  }
  rowptr[n] = (uint32_t)k;
  return k;
}

}  // namespace

extern "C" {

// Reference pattern of `map f to E` over an edge set E(V,...,V) with `card`
// endpoints.  Returns nnz, or -1 when `cap` is too small, -2 on bad card.
int64_t ref_pattern(int32_t n, const int32_t *ep, int64_t nE, int32_t card,
                    uint32_t *rowptr, uint32_t *colidx, int64_t cap) {
  simit::Set V;
  std::vector<ElementRef> vr;
  vr.reserve(n);
  for (int32_t i = 0; i < n; ++i) vr.push_back(V.add());
  switch (card) {
    case 1: {
      simit::Set E(V);
      for (int64_t i = 0; i < nE; ++i) E.add(vr[ep[i]]);
      return build_with(V, vr, E, ep, nE, card, rowptr, colidx, cap);
    }
    case 2: {
      simit::Set E(V, V);
      for (int64_t i = 0; i < nE; ++i) E.add(vr[ep[2 * i]], vr[ep[2 * i + 1]]);
      return build_with(V, vr, E, ep, nE, card, rowptr, colidx, cap);
    }
    case 3: {
      simit::Set E(V, V, V);
      for (int64_t i = 0; i < nE; ++i)
        E.add(vr[ep[3 * i]], vr[ep[3 * i + 1]], vr[ep[3 * i + 2]]);
      return build_with(V, vr, E, ep, nE, card, rowptr, colidx, cap);
    }
    case 4: {
      simit::Set E(V, V, V, V);
      for (int64_t i = 0; i < nE; ++i)
        E.add(vr[ep[4 * i]], vr[ep[4 * i + 1]], vr[ep[4 * i + 2]],
              vr[ep[4 * i + 3]]);
      return build_with(V, vr, E, ep, nE, card, rowptr, colidx, cap);
    }
    default:
      return -2;
  }
}

// The reference's own Link::ev / Link::ve indices (src/path_indices.cpp:
// 207-276) and the And of the two between different vertex sets, for an
// edge set whose endpoint k lies in vertex set set_of[k] (0 -> V0, 1 -> V1),
// as src/path_expression_analysis.cpp:80-105 builds them for tensor[E,X],
// tensor[X,E] and matrix[Xr,Xc].  kind 0: ev (rows E, columns set xc);
// 1: ve (rows set xr, columns E); 2: ∃e.(v-e ∧ e-u), v in xr, u in xc.
// Returns nnz, -1 when cap is too small, -2 on a bad card.
static int64_t ref_incidence_build(int kind, simit::Set &V0, simit::Set &V1, simit::Set &E,
                                   int32_t xr, int32_t xc, uint32_t *rowptr,
                                   uint32_t *colidx, int64_t cap) {
  PathIndexBuilder builder;
  builder.bind("V0", &V0);
  builder.bind("V1", &V1);
  builder.bind("E", &E);
  Var e("e", pe::Set("E"));
  Var v("v", pe::Set(xr ? "V1" : "V0"));
  Var u("u", pe::Set(xc ? "V1" : "V0"));
  PathExpression pexpr;
  if (kind == 0) pexpr = Link::make(e, u, Link::ev);
  else if (kind == 1) pexpr = Link::make(v, e, Link::ve);
  else
    pexpr = And::make({v, u}, {{QuantifiedVar::Exist, e}}, Link::make(v, e, Link::ve)(v, e),
                      Link::make(e, u, Link::ev)(e, u));
  PathIndex pidx = builder.buildSegmented(pexpr, 0);
  const int64_t n = (int64_t)pidx.numElements();
  int64_t k = 0;
  for (int64_t r = 0; r < n; ++r) {
    rowptr[r] = (uint32_t)k;
    for (unsigned c : pidx.neighbors((unsigned)r)) {
      if (k >= cap) return -1;
      colidx[k++] = c;
    }
  }
  rowptr[n] = (uint32_t)k;
  return k;
}

int64_t ref_incidence(int kind, int32_t n0, int32_t n1, int32_t card, const int32_t *set_of,
                      const int32_t *ep, int64_t nE, int32_t xr, int32_t xc, uint32_t *rowptr,
                      uint32_t *colidx, int64_t cap) {
  simit::Set V0, V1;
  std::vector<ElementRef> r0, r1;
  for (int32_t i = 0; i < n0; ++i) r0.push_back(V0.add());
  for (int32_t i = 0; i < n1; ++i) r1.push_back(V1.add());
  simit::Set *S[5];
  for (int k = 0; k < card && k < 5; ++k) S[k] = set_of[k] ? &V1 : &V0;
  auto at = [&](int64_t e, int k) -> ElementRef & {
    return set_of[k] ? r1[ep[e * card + k]] : r0[ep[e * card + k]];
  };
  switch (card) {
    case 2: {
      simit::Set E(*S[0], *S[1]);
      for (int64_t i = 0; i < nE; ++i) E.add(at(i, 0), at(i, 1));
      return ref_incidence_build(kind, V0, V1, E, xr, xc, rowptr, colidx, cap);
    }
    case 3: {
      simit::Set E(*S[0], *S[1], *S[2]);
      for (int64_t i = 0; i < nE; ++i) E.add(at(i, 0), at(i, 1), at(i, 2));
      return ref_incidence_build(kind, V0, V1, E, xr, xc, rowptr, colidx, cap);
    }
    case 4: {
      simit::Set E(*S[0], *S[1], *S[2], *S[3]);
      for (int64_t i = 0; i < nE; ++i) E.add(at(i, 0), at(i, 1), at(i, 2), at(i, 3));
      return ref_incidence_build(kind, V0, V1, E, xr, xc, rowptr, colidx, cap);
    }
    case 5: {
      simit::Set E(*S[0], *S[1], *S[2], *S[3], *S[4]);
      for (int64_t i = 0; i < nE; ++i)
        E.add(at(i, 0), at(i, 1), at(i, 2), at(i, 3), at(i, 4));
      return ref_incidence_build(kind, V0, V1, E, xr, xc, rowptr, colidx, cap);
    }
    default:
      return -2;
  }
}

// The reference runtime's slot search `loc` (src/runtime.cpp:19-23) applied
// per element and endpoint pair (i, j) in the order gatherVVLocs emits the
// calls (src/inline.cpp:544-552): slots[e*card*card + i*card + j].
void ref_slots(const int32_t *ep, int64_t nE, int32_t card,
               const uint32_t *rowptr, const uint32_t *colidx,
               uint32_t *slots) {
  for (int64_t e = 0; e < nE; ++e)
    for (int i = 0; i < card; ++i)
      for (int j = 0; j < card; ++j)
        slots[(e * card + i) * card + j] = (uint32_t)loc(
            ep[e * card + i], ep[e * card + j], (int *)rowptr, (int *)colidx);
}

}  // extern "C"
