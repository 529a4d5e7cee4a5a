// Incidence matrices of an edge set over one of its vertex sets, the
// reference's two non-square assembly patterns (src/path_expression_analysis
// .cpp:95-105):
//   EV, tensor[E,V]: Link::ev (src/path_indices.cpp:207-246) -- row e lists
//       the element's endpoints in that vertex set in endpoint order,
//       repeats kept;
//   VE, tensor[V,E]: Link::ve (:248-276) -- row v lists the elements that
//       have v among those endpoints, ascending, once per listing.
// A `map` whose element function writes A(p(k), e) or A(e, p(k)) adds the
// value into the slot `loc` finds, the first one of that (row, column) in
// its row (src/runtime.cpp:19-23), so the slot of a repeated endpoint's
// second listing stays zero.  Every slot belongs to one element, so the
// assembly is a thread per (element, listing) with no accumulation across
// elements; a listing sums the blocks of its element's repeats of the same
// vertex in ascending k, from zero, as the reference's `+=`s do.
#include <stdint.h>

#include "sg_internal.cuh"

namespace sg {
namespace {

__global__ void k_ev_rowptr(int64_t nE, int32_t npos, uint32_t *__restrict__ rowptr) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e <= nE;
       e += (int64_t)gridDim.x * blockDim.x)
    rowptr[e] = (uint32_t)(e * npos);
}

__global__ void k_ev_colidx(int64_t m, int32_t n, const int32_t *__restrict__ sel,
                            uint32_t *__restrict__ colidx, int *err) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = sel[t];
    if (v < 0 || v >= n) atomicCAS(err, 0, (int)DEV_BAD_ENDPOINT);
    colidx[t] = (uint32_t)v;
  }
}

// In place over the sorted incidence (listing t = e*npos + k in colidx):
// the VE column t / npos and the slot of every listing.  Each slot is read
// and written by one thread only.
__global__ void k_ve_cols(int64_t m, int32_t npos, uint32_t *__restrict__ colidx,
                          uint32_t *__restrict__ slot_of, int *err) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < m;
       q += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t t = colidx[q];
    if (t >= (uint64_t)m) {  // cannot happen for a built incidence; never write out of range
      atomicCAS(err, 0, (int)DEV_BAD_ENDPOINT);
      continue;
    }
    colidx[q] = t / (uint32_t)npos;
    slot_of[t] = (uint32_t)q;
  }
}

template <typename T>
__global__ void k_assemble_incidence(int64_t m, int32_t npos, int bb, int ve,
                                     const int32_t *__restrict__ sel,
                                     const uint32_t *__restrict__ slot_of,
                                     const T *__restrict__ eb, T *__restrict__ vals, int *err) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / npos;
    const int k = (int)(t - e * npos);
    const int32_t *p = sel + e * npos;
    const int32_t v = p[k];
    bool first = true;
    for (int j = 0; j < k; ++j) first = first && p[j] != v;
    const size_t slot = ve ? slot_of[t] : (size_t)t;
    if (slot >= (size_t)m) {  // a slot map not made by sg_incidence_pattern
      atomicCAS(err, 0, (int)DEV_SLOT_MISSING);
      continue;
    }
    for (int w = 0; w < bb; ++w) {
      T s = T(0);
      if (first)
        for (int j = k; j < npos; ++j)
          if (p[j] == v) s = s + eb[(size_t)(e * npos + j) * bb + w];
      vals[slot * bb + w] = s;
    }
  }
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" {

int sg_incidence_pattern(sg_ctx *h, int kind, int32_t n, int64_t nE, int32_t npos,
                         const int32_t *sel, uint32_t *rowptr, uint32_t *colidx,
                         uint32_t *slot_of) {
  Ctx *c = as_ctx(h);
  SG_REQUIRE(c && rowptr, "sg_incidence_pattern: null argument");
  SG_REQUIRE(kind == SG_INCIDENCE_EV || kind == SG_INCIDENCE_VE,
             "sg_incidence_pattern: kind %d", kind);
  SG_REQUIRE(n >= 0 && nE >= 0 && npos >= 1 && npos <= 16,
             "sg_incidence_pattern: n %d nE %lld npos %d", n, (long long)nE, npos);
  const int64_t m = nE * npos;
  SG_REQUIRE(m < 0xffffffffLL, "sg_incidence_pattern: %lld listings", (long long)m);
  SG_REQUIRE(m == 0 || (sel && colidx), "sg_incidence_pattern: null array");
  if (kind == SG_INCIDENCE_EV) {
    k_ev_rowptr<<<grid_for(c, nE + 1, 256, 8), 256, 0, c->stream>>>(nE, npos, rowptr);
    SG_CHECK_LAUNCH();
    if (m > 0) {
      k_ev_colidx<<<grid_for(c, m, 256, 8), 256, 0, c->stream>>>(m, n, sel, colidx, c->d_err);
      SG_CHECK_LAUNCH();
    }
    return check_device_error(c, "sg_incidence_pattern");
  }
  SG_REQUIRE(m == 0 || slot_of, "sg_incidence_pattern: VE needs slot_of");
  if (m == 0) {
    SG_CHECK_CUDA(cudaMemsetAsync(rowptr, 0, (size_t)(n + 1) * 4, c->stream));
    return SG_OK;
  }
  // the sorted incidence goes straight into colidx (sg_incidence_build uses
  // the context's scratch arena itself, so nothing here may hold scratch)
  SG_TRY(sg_incidence_build(h, n, sel, nE, npos, rowptr, colidx));
  k_ve_cols<<<grid_for(c, m, 256, 8), 256, 0, c->stream>>>(m, npos, colidx, slot_of, c->d_err);
  SG_CHECK_LAUNCH();
  return check_device_error(c, "sg_incidence_pattern");
}

int sg_assemble_incidence(sg_ctx *h, int kind, int64_t nE, int32_t npos, const int32_t *sel,
                          const uint32_t *slot_of, int dtype, int32_t bs, const void *eb,
                          void *vals) {
  Ctx *c = as_ctx(h);
  SG_REQUIRE(c, "sg_assemble_incidence: null context");
  SG_REQUIRE(kind == SG_INCIDENCE_EV || kind == SG_INCIDENCE_VE,
             "sg_assemble_incidence: kind %d", kind);
  SG_REQUIRE(nE >= 0 && npos >= 1 && npos <= 16 && bs >= 1 && bs <= 4,
             "sg_assemble_incidence: nE %lld npos %d bs %d", (long long)nE, npos, bs);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_assemble_incidence: dtype %d", dtype);
  const int64_t m = nE * npos;
  if (m == 0) return SG_OK;
  SG_REQUIRE(sel && eb && vals && (kind == SG_INCIDENCE_EV || slot_of),
             "sg_assemble_incidence: null array");
  const int g = grid_for(c, m, 256, 8);
  const int ve = kind == SG_INCIDENCE_VE;
  if (dtype == SG_F64)
    k_assemble_incidence<double><<<g, 256, 0, c->stream>>>(
        m, npos, bs * bs, ve, sel, slot_of, (const double *)eb, (double *)vals, c->d_err);
  else
    k_assemble_incidence<float><<<g, 256, 0, c->stream>>>(
        m, npos, bs * bs, ve, sel, slot_of, (const float *)eb, (float *)vals, c->d_err);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // extern "C"
