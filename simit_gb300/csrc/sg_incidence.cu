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
  DeviceGuard dg_(c);
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
  DeviceGuard dg_(c);
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

// ---------------------------------------------------------------------------
// Rectangular vertex-vertex pattern ∃e.(v-e ∧ e-u) between two vertex sets of
// one edge set (src/path_expression_analysis.cpp:80-92 with v and u in
// different sets): row v of the row set lists, sorted and unique, the column
// set's endpoints of every element that has v among its row-set endpoints.
// A thread per row gathers the candidates through the row set's incidence
// (sg_incidence_build over sel_r) into a sorted local list.
// ---------------------------------------------------------------------------
namespace sg {
namespace {

constexpr int RECT_CAP = 64;  // columns of one row (DEV_ROW_TOO_LONG beyond)

__device__ int rect_row(uint32_t v, const uint32_t *__restrict__ ve_ptr,
                        const uint32_t *__restrict__ ve_idx, int32_t npos_r, int32_t npos_c,
                        const int32_t *__restrict__ sel_c, int32_t nc, uint32_t *cols,
                        int *err) {
  int len = 0;
  for (uint32_t q = ve_ptr[v]; q < ve_ptr[v + 1]; ++q) {
    const uint32_t e = ve_idx[q] / (uint32_t)npos_r;
    for (int j = 0; j < npos_c; ++j) {
      const int32_t u = sel_c[(size_t)e * npos_c + j];
      if (u < 0 || u >= nc) {
        atomicCAS(err, 0, (int)DEV_BAD_ENDPOINT);
        continue;
      }
      int pos = len;  // insertion into the sorted unique list
      while (pos > 0 && cols[pos - 1] > (uint32_t)u) --pos;
      if (pos > 0 && cols[pos - 1] == (uint32_t)u) continue;
      if (len == RECT_CAP) {
        atomicCAS(err, 0, (int)DEV_ROW_TOO_LONG);
        return len;
      }
      for (int i = len; i > pos; --i) cols[i] = cols[i - 1];
      cols[pos] = (uint32_t)u;
      ++len;
    }
  }
  return len;
}

__global__ void k_rect_count(int32_t nr, const uint32_t *__restrict__ ve_ptr,
                             const uint32_t *__restrict__ ve_idx, int32_t npos_r,
                             int32_t npos_c, const int32_t *__restrict__ sel_c, int32_t nc,
                             uint32_t *__restrict__ cnt, int *err) {
  uint32_t cols[RECT_CAP];
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nr;
       v += (int64_t)gridDim.x * blockDim.x)
    cnt[v] = (uint32_t)rect_row((uint32_t)v, ve_ptr, ve_idx, npos_r, npos_c, sel_c, nc, cols,
                                err);
}

__global__ void k_rect_fill(int32_t nr, const uint32_t *__restrict__ ve_ptr,
                            const uint32_t *__restrict__ ve_idx, int32_t npos_r, int32_t npos_c,
                            const int32_t *__restrict__ sel_c, int32_t nc,
                            const uint32_t *__restrict__ rowptr, uint32_t *__restrict__ colidx,
                            int *err) {
  uint32_t cols[RECT_CAP];
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nr;
       v += (int64_t)gridDim.x * blockDim.x) {
    const int len = rect_row((uint32_t)v, ve_ptr, ve_idx, npos_r, npos_c, sel_c, nc, cols, err);
    const uint32_t r0 = rowptr[v];
    if ((int64_t)len != (int64_t)rowptr[v + 1] - r0) {
      atomicCAS(err, 0, (int)DEV_SLOT_MISSING);
      continue;
    }
    for (int i = 0; i < len; ++i) colidx[r0 + i] = cols[i];
  }
}

// Row owner: zero the row, then for its listings (e ascending, then k) and
// the element's column endpoints j, add block (e, k, j) into its slot.
template <typename T>
__global__ void k_rect_assemble(int32_t nr, const uint32_t *__restrict__ ve_ptr,
                                const uint32_t *__restrict__ ve_idx, int32_t npos_r,
                                int32_t npos_c, const int32_t *__restrict__ sel_c,
                                const uint32_t *__restrict__ rowptr,
                                const uint32_t *__restrict__ colidx, int bb,
                                const T *__restrict__ eb, T *__restrict__ vals, int *err) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nr;
       v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t r0 = rowptr[v], r1 = rowptr[v + 1];
    for (size_t q = (size_t)r0 * bb; q < (size_t)r1 * bb; ++q) vals[q] = T(0);
    for (uint32_t it = ve_ptr[v]; it < ve_ptr[v + 1]; ++it) {
      const uint32_t t = ve_idx[it];  // e*npos_r + k
      const uint32_t e = t / (uint32_t)npos_r;
      for (int j = 0; j < npos_c; ++j) {
        const uint32_t u = (uint32_t)sel_c[(size_t)e * npos_c + j];
        uint32_t lo = r0, hi = r1;
        while (lo < hi) {
          const uint32_t m = lo + ((hi - lo) >> 1);
          if (colidx[m] < u) lo = m + 1;
          else hi = m;
        }
        if (lo == r1 || colidx[lo] != u) {
          atomicCAS(err, 0, (int)DEV_SLOT_MISSING);
          continue;
        }
        const T *b = eb + ((size_t)t * npos_c + j) * bb;
        for (int w = 0; w < bb; ++w) vals[(size_t)lo * bb + w] += b[w];
      }
    }
  }
}

}  // namespace
}  // namespace sg

extern "C" {

int sg_pattern_rect(sg_ctx *h, int32_t nr, int32_t nc, int64_t nE, int32_t npos_r,
                    int32_t npos_c, const int32_t *sel_c, const uint32_t *ve_ptr,
                    const uint32_t *ve_idx, uint32_t *rowptr, uint32_t *colidx,
                    int64_t *h_nnzb) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && rowptr && h_nnzb && ve_ptr, "sg_pattern_rect: null argument");
  SG_REQUIRE(nr >= 0 && nc >= 0 && nE >= 0 && npos_r >= 1 && npos_r <= 16 && npos_c >= 1 &&
                 npos_c <= 16,
             "sg_pattern_rect: nr %d nc %d nE %lld npos %d/%d", nr, nc, (long long)nE, npos_r,
             npos_c);
  SG_REQUIRE(nE == 0 || (sel_c && ve_idx), "sg_pattern_rect: null array");
  const int g = grid_for(c, nr, 128, 8);
  if (!colidx) {  // count pass: rowptr and nnzb
    Scratch s(c);
    SG_TRY(s.reserve(Scratch::bytes_for((size_t)nr + 1, 4) + scan_scratch_bytes(nr) + 512));
    uint32_t *cnt = s.alloc<uint32_t>((size_t)nr + 1);
    if (nr > 0) {
      k_rect_count<<<g, 128, 0, c->stream>>>(nr, ve_ptr, ve_idx, npos_r, npos_c, sel_c, nc, cnt,
                                            c->d_err);
      SG_CHECK_LAUNCH();
    }
    SG_TRY(exclusive_scan_u32(c, s, cnt, rowptr, nr));
    SG_TRY(check_device_error(c, "sg_pattern_rect"));
    uint32_t tot = 0;
    SG_CHECK_CUDA(cudaMemcpyAsync(&tot, rowptr + nr, 4, cudaMemcpyDeviceToHost, c->stream));
    SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
    *h_nnzb = tot;
    return SG_OK;
  }
  if (nr > 0) {
    k_rect_fill<<<g, 128, 0, c->stream>>>(nr, ve_ptr, ve_idx, npos_r, npos_c, sel_c, nc, rowptr,
                                         colidx, c->d_err);
    SG_CHECK_LAUNCH();
  }
  return check_device_error(c, "sg_pattern_rect");
}

int sg_assemble_rect(sg_ctx *h, int32_t nr, int32_t npos_r, int32_t npos_c,
                     const int32_t *sel_c, const uint32_t *ve_ptr, const uint32_t *ve_idx,
                     const uint32_t *rowptr, const uint32_t *colidx, int dtype, int32_t bs,
                     const void *eb, void *vals) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && ve_ptr && rowptr, "sg_assemble_rect: null argument");
  SG_REQUIRE(nr >= 0 && npos_r >= 1 && npos_r <= 16 && npos_c >= 1 && npos_c <= 16 && bs >= 1 &&
                 bs <= 4,
             "sg_assemble_rect: nr %d npos %d/%d bs %d", nr, npos_r, npos_c, bs);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_assemble_rect: dtype %d", dtype);
  if (nr == 0) return SG_OK;
  const int g = grid_for(c, nr, 128, 8);
  if (dtype == SG_F64)
    k_rect_assemble<double><<<g, 128, 0, c->stream>>>(nr, ve_ptr, ve_idx, npos_r, npos_c, sel_c,
                                                     rowptr, colidx, bs * bs,
                                                     (const double *)eb, (double *)vals,
                                                     c->d_err);
  else
    k_rect_assemble<float><<<g, 128, 0, c->stream>>>(nr, ve_ptr, ve_idx, npos_r, npos_c, sel_c,
                                                    rowptr, colidx, bs * bs, (const float *)eb,
                                                    (float *)vals, c->d_err);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // extern "C"
