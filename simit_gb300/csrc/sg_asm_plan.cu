// Assembly plans: the element colouring and the inverse slot map.
//
// Inverse slot map (the element-blocks + slot-gather plan): for every
// matrix slot the list of element blocks (e*card + i)*card + j whose slot it
// is, ascending (ascending element, then i, j), as CSR (slot_src_ptr,
// slot_src).  Built by counting, a scan, scattering with per-slot cursors
// and a per-slot insertion sort, so the lists do not depend on timing.
//
// Element colouring (the coloured plan):
// Two elements that share a vertex write blocks of the same matrix rows, so
// elements are coloured such that no two of one colour share a vertex; the
// assembly then adds each colour's element blocks into their precomputed
// slots with plain read-modify-writes (no atomics), colour after colour, in
// a fixed order (deterministic results).  The reference has no counterpart:
// its GPU backend adds element blocks with float atomics
// (src/backend/gpu/gpu_backend.cpp:788-846) and its CPU backend runs the
// element loop serially (src/inline.cpp:690-888).
//
// Colouring: Jones-Plassmann.  Every element gets a fixed pseudo-random
// priority (a hash of its index, ties by index).  Each round, every
// uncoloured element that outranks all of its uncoloured neighbours (the
// elements on its vertices' incidence lists) takes the smallest colour none
// of its coloured neighbours has.  Rounds read the colours of the previous
// round and write a second array, so the result does not depend on thread
// timing.  Elements are then listed colour by colour, ascending index within
// a colour.
#include <utility>

#include "sg_internal.cuh"

namespace sg {

constexpr int MAX_COLORS = SG_MAX_COLORS;

__device__ __forceinline__ uint32_t color_prio(uint32_t e) {
  uint32_t h = e * 0x9E3779B1u;
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}

// One round: cur -> nxt.  A coloured element keeps its colour; an
// uncoloured one takes a colour when it outranks every uncoloured
// neighbour, else stays -1 and is counted in *left.
__global__ void k_jp_round(int64_t nE, int32_t card, const int32_t *__restrict__ ep,
                           const uint32_t *__restrict__ ve_ptr,
                           const uint32_t *__restrict__ ve_idx, const int32_t *__restrict__ cur,
                           int32_t *__restrict__ nxt, unsigned long long *left, int *err) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nE;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int32_t c0 = cur[e];
    if (c0 >= 0) {
      nxt[e] = c0;
      continue;
    }
    const uint32_t pe = color_prio((uint32_t)e);
    bool top = true;
    uint64_t f0 = 0, f1 = 0;
    for (int i = 0; i < card && top; ++i) {
      const int32_t v = ep[e * card + i];
      for (uint32_t t = ve_ptr[v]; t < ve_ptr[v + 1]; ++t) {
        const uint32_t e2 = ve_idx[t] / (uint32_t)card;
        if (e2 == (uint32_t)e) continue;
        const int32_t c2 = cur[e2];
        if (c2 < 0) {
          const uint32_t p2 = color_prio(e2);
          if (p2 > pe || (p2 == pe && e2 > (uint32_t)e)) {
            top = false;
            break;
          }
        } else if (c2 < 64) {
          f0 |= 1ull << c2;
        } else {
          f1 |= 1ull << (c2 - 64);
        }
      }
    }
    int32_t col = -1;
    if (top) {
      if (~f0) col = __ffsll((long long)~f0) - 1;
      else if (~f1) col = 64 + __ffsll((long long)~f1) - 1;
      else atomicCAS(err, 0, DEV_TOO_MANY_COLORS);
    }
    nxt[e] = col;
    if (col < 0) atomicAdd(left, 1ull);
  }
}

__global__ void k_color_flags(int64_t nE, const int32_t *__restrict__ col, int32_t c,
                              uint32_t *__restrict__ flag) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nE;
       e += (int64_t)gridDim.x * blockDim.x)
    flag[e] = col[e] == c ? 1u : 0u;
}

__global__ void k_color_scatter(int64_t nE, const uint32_t *__restrict__ flag,
                                const uint32_t *__restrict__ pos, uint32_t base,
                                uint32_t *__restrict__ order) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nE;
       e += (int64_t)gridDim.x * blockDim.x)
    if (flag[e]) order[base + pos[e]] = (uint32_t)e;
}

__global__ void k_src_count(int64_t m, const uint32_t *__restrict__ slots, int64_t nnzb,
                            uint32_t *__restrict__ cnt, int *err) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < m;
       b += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t q = slots[b];
    if ((int64_t)q >= nnzb) {
      atomicCAS(err, 0, DEV_SLOT_MISSING);
      continue;
    }
    atomicAdd(&cnt[q], 1u);
  }
}

__global__ void k_src_scatter(int64_t m, const uint32_t *__restrict__ slots, int64_t nnzb,
                              const uint32_t *__restrict__ sptr, uint32_t *__restrict__ cursor,
                              uint32_t *__restrict__ src) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < m;
       b += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t q = slots[b];
    if ((int64_t)q >= nnzb) continue;
    src[sptr[q] + atomicAdd(&cursor[q], 1u)] = (uint32_t)b;
  }
}

__global__ void k_src_sort(int64_t nnzb, const uint32_t *__restrict__ sptr,
                           uint32_t *__restrict__ src) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnzb;
       q += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t k0 = sptr[q], k1 = sptr[q + 1];
    for (uint32_t k = k0 + 1; k < k1; ++k) {
      const uint32_t v = src[k];
      uint32_t p = k;
      while (p > k0 && src[p - 1] > v) {
        src[p] = src[p - 1];
        --p;
      }
      src[p] = v;
    }
  }
}

}  // namespace sg

using namespace sg;

extern "C" {

int sg_slot_sources(sg_ctx *h, const sg_mesh *m, uint32_t *slot_src_ptr, uint32_t *slot_src) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && m && slot_src_ptr, "sg_slot_sources: null argument");
  const int64_t mm = m->nE * (int64_t)m->card * m->card;
  SG_REQUIRE(mm == 0 || (m->slots && slot_src), "sg_slot_sources: the mesh needs its slots");
  SG_REQUIRE(mm < (int64_t)0xffffffffll, "sg_slot_sources: nE*card*card must fit in uint32");
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(m->nnzb + 1, 4) * 2 + scan_scratch_bytes(m->nnzb) + 512));
  uint32_t *cnt = s.alloc<uint32_t>(m->nnzb + 1);
  uint32_t *cursor = s.alloc<uint32_t>(m->nnzb + 1);
  SG_CHECK_CUDA(cudaMemsetAsync(cnt, 0, (m->nnzb + 1) * 4, c->stream));
  SG_CHECK_CUDA(cudaMemsetAsync(cursor, 0, (m->nnzb + 1) * 4, c->stream));
  const int g = grid_for(c, mm, 256, 8);
  if (mm > 0) {
    k_src_count<<<g, 256, 0, c->stream>>>(mm, m->slots, m->nnzb, cnt, c->d_err);
    SG_CHECK_LAUNCH();
  }
  SG_TRY(exclusive_scan_u32(c, s, cnt, slot_src_ptr, m->nnzb));
  SG_TRY(check_device_error(c, "sg_slot_sources"));
  if (mm == 0) return SG_OK;
  k_src_scatter<<<g, 256, 0, c->stream>>>(mm, m->slots, m->nnzb, slot_src_ptr, cursor, slot_src);
  SG_CHECK_LAUNCH();
  k_src_sort<<<grid_for(c, m->nnzb, 256, 8), 256, 0, c->stream>>>(m->nnzb, slot_src_ptr,
                                                                  slot_src);
  SG_CHECK_LAUNCH();
  return check_device_error(c, "sg_slot_sources");
}

int sg_element_coloring(sg_ctx *h, const sg_mesh *m, uint32_t *color_order, int32_t *color_ptr,
                        int32_t *h_ncolors) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && m && color_ptr && h_ncolors, "sg_element_coloring: null argument");
  SG_REQUIRE(m->nE == 0 || (color_order && m->endpoints && m->ve_ptr && m->ve_idx),
             "sg_element_coloring: the mesh needs endpoints and its incidence");
  SG_REQUIRE(m->card >= 1 && m->nE < (int64_t)0xffffffffll / m->card,
             "sg_element_coloring: nE*card must fit in uint32");
  const int64_t nE = m->nE;
  *h_ncolors = 0;
  color_ptr[0] = 0;
  if (nE == 0) return SG_OK;
  Scratch s(c);
  // two colour arrays, flags and positions, and the scratch of one scan per
  // colour (each scan's bump allocations stay live until the call returns)
  SG_TRY(s.reserve(Scratch::bytes_for(nE + 1, 4) * 4 +
                   (size_t)(MAX_COLORS + 1) * scan_scratch_bytes(nE) + 1024));
  int32_t *ca = s.alloc<int32_t>(nE);
  int32_t *cb = s.alloc<int32_t>(nE);
  unsigned long long *left = s.alloc<unsigned long long>(1);
  SG_CHECK_CUDA(cudaMemsetAsync(ca, 0xff, nE * 4, c->stream));  // all -1
  const int grid = grid_for(c, nE, 256, 8);
  int32_t *cur = ca, *nxt = cb;
  for (int round = 0;; ++round) {
    SG_REQUIRE(round < 100000, "sg_element_coloring: no progress");
    SG_CHECK_CUDA(cudaMemsetAsync(left, 0, 8, c->stream));
    k_jp_round<<<grid, 256, 0, c->stream>>>(nE, m->card, m->endpoints, m->ve_ptr, m->ve_idx,
                                            cur, nxt, left, c->d_err);
    SG_CHECK_LAUNCH();
    SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, left, 8, cudaMemcpyDeviceToHost, c->stream));
    SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
    SG_TRY(check_device_error(c, "sg_element_coloring"));
    std::swap(cur, nxt);
    if (*(unsigned long long *)c->h_stage == 0) break;
  }
  // the elements of each colour in ascending index
  uint32_t *flag = s.alloc<uint32_t>(nE + 1);
  uint32_t *pos = s.alloc<uint32_t>(nE + 1);
  uint32_t base = 0;
  int nc = 0;
  for (int col = 0; col < MAX_COLORS; ++col) {
    k_color_flags<<<grid, 256, 0, c->stream>>>(nE, cur, col, flag);
    SG_CHECK_LAUNCH();
    SG_TRY(exclusive_scan_u32(c, s, flag, pos, nE));
    SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, pos + nE, 4, cudaMemcpyDeviceToHost, c->stream));
    SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
    const uint32_t cnt = *(uint32_t *)c->h_stage;
    if (cnt == 0) break;  // colours are taken smallest first: none above an empty one
    k_color_scatter<<<grid, 256, 0, c->stream>>>(nE, flag, pos, base, color_order);
    SG_CHECK_LAUNCH();
    base += cnt;
    color_ptr[++nc] = (int32_t)base;
  }
  SG_REQUIRE(base == (uint32_t)nE, "sg_element_coloring: %u of %lld elements ordered", base,
             (long long)nE);
  *h_ncolors = nc;
  return SG_OK;
}

}  // extern "C"
