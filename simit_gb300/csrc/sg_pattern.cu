// Pattern construction on the GPU: vertex incidence, blocked-CSR rows of
// ∃e∈E.(v-e ∧ e-u), and the element-to-slot map.
//
// Output is bit-identical to the reference's PathIndexBuilder
// (src/path_indices.cpp:148-531): row v is the sorted set of every endpoint
// of every element incident on v (empty when v has none), and slot (e,i,j)
// is the position `loc` (src/runtime.cpp:19-23) finds for
// (ep[e,i], ep[e,j]).
//
// Design: no std::set and no global sort.  Incidences are bucketed by vertex
// with integer atomics (counts only), and each vertex's bucket is then sorted
// by (e*card + i) inside one warp, so every result is deterministic.  Row
// columns come from a per-warp shared-memory bitonic sort + unique of the
// bucket's endpoints; slots from a binary search of the sorted row.
#include "sg_internal.cuh"

namespace sg {

__device__ __forceinline__ void dev_fail(int *err, int code) {
  atomicCAS(err, 0, code);
}

__global__ void inc_count(const int32_t *ep, int64_t m, int32_t n,
                          uint32_t *cnt, int *err) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x) {
    int32_t v = ep[t];
    if (v < 0 || v >= n) {
      dev_fail(err, DEV_BAD_ENDPOINT);
      continue;
    }
    atomicAdd(&cnt[v], 1u);
  }
}

__global__ void inc_fill(const int32_t *ep, int64_t m, int32_t n,
                         uint32_t *cursor, uint32_t *ve_idx) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x) {
    int32_t v = ep[t];
    if (v < 0 || v >= n) continue;
    uint32_t pos = atomicAdd(&cursor[v], 1u);
    ve_idx[pos] = (uint32_t)t;
  }
}

__global__ void max_u32_diff(const uint32_t *ptr, int32_t n, uint32_t *out) {
  uint32_t m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, ptr[i + 1] - ptr[i]);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Warp-cooperative bitonic sort (ascending) of `len` (a power of two, >= 32)
// keys in shared memory.
__device__ void warp_bitonic_sort(uint32_t *s, int len) {
  const int lane = threadIdx.x & 31;
  for (int k = 2; k <= len; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < len; i += 32) {
        int ixj = i ^ j;
        if (ixj > i) {
          uint32_t a = s[i], b = s[ixj];
          bool up = ((i & k) == 0);
          if ((a > b) == up) {
            s[i] = b;
            s[ixj] = a;
          }
        }
      }
      __syncwarp();
    }
  }
}

__device__ __forceinline__ int pow2_at_least(int x) {
  int p = 32;
  while (p < x) p <<= 1;
  return p;
}

// One warp per vertex: sort its incidence bucket ascending.
__global__ void inc_sort(const uint32_t *ve_ptr, uint32_t *ve_idx, int32_t n,
                         int cap, int *err) {
  extern __shared__ uint32_t smem[];
  const int wpb = blockDim.x >> 5;
  uint32_t *s = smem + (threadIdx.x >> 5) * cap;
  const int lane = threadIdx.x & 31;
  for (int64_t v = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); v < n;
       v += (int64_t)gridDim.x * wpb) {
    const uint32_t b = ve_ptr[v], e = ve_ptr[v + 1];
    const int len = (int)(e - b);
    if (len <= 1) continue;
    if (len <= 32) {  // register bitonic
      uint32_t key = lane < len ? ve_idx[b + lane] : 0xffffffffu;
      for (int k = 2; k <= 32; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
          uint32_t other = __shfl_xor_sync(0xffffffffu, key, j);
          bool up = ((lane & k) == 0);
          bool lower = ((lane & j) == 0);
          uint32_t mn = min(key, other), mx = max(key, other);
          key = (lower == up) ? mn : mx;
        }
      if (lane < len) ve_idx[b + lane] = key;
      continue;
    }
    if (len > cap) {
      if (lane == 0) dev_fail(err, DEV_ROW_TOO_LONG);
      continue;
    }
    const int p2 = pow2_at_least(len);
    for (int i = lane; i < p2; i += 32) s[i] = i < len ? ve_idx[b + i] : 0xffffffffu;
    __syncwarp();
    warp_bitonic_sort(s, p2);
    for (int i = lane; i < len; i += 32) ve_idx[b + i] = s[i];
    __syncwarp();
  }
}

// One warp per vertex: gather the endpoints of every incident element, sort,
// unique.  Pass 0 writes the unique count to rowcnt[v]; pass 1 writes the
// columns at colidx[rowptr[v]...].
__global__ void rows_build(const int32_t *ep, int32_t card, const uint32_t *ve_ptr,
                           const uint32_t *ve_idx, int32_t n, int cap, int pass,
                           uint32_t *rowcnt, const uint32_t *rowptr,
                           uint32_t *colidx, int *err) {
  extern __shared__ uint32_t smem[];
  const int wpb = blockDim.x >> 5;
  uint32_t *s = smem + (threadIdx.x >> 5) * cap;
  const int lane = threadIdx.x & 31;
  for (int64_t v = (int64_t)blockIdx.x * wpb + (threadIdx.x >> 5); v < n;
       v += (int64_t)gridDim.x * wpb) {
    const uint32_t b = ve_ptr[v], e = ve_ptr[v + 1];
    const int len = (int)(e - b) * card;
    if (len == 0) {
      if (pass == 0 && lane == 0) rowcnt[v] = 0;
      continue;
    }
    if (len > cap) {
      if (lane == 0) {
        dev_fail(err, DEV_ROW_TOO_LONG);
        if (pass == 0) rowcnt[v] = 0;
      }
      continue;
    }
    const int p2 = pow2_at_least(len);
    for (int i = lane; i < p2; i += 32) {
      uint32_t val = 0xffffffffu;
      if (i < len) {
        const uint32_t t = ve_idx[b + i / card];
        const uint32_t el = t / (uint32_t)card;
        val = (uint32_t)ep[(int64_t)el * card + (i % card)];
      }
      s[i] = val;
    }
    __syncwarp();
    warp_bitonic_sort(s, p2);
    // unique: keep s[i] when i == 0 or s[i] != s[i-1]
    uint32_t out = 0;
    const uint32_t base = (pass == 1) ? rowptr[v] : 0;
    for (int i0 = 0; i0 < len; i0 += 32) {
      const int i = i0 + lane;
      bool keep = (i < len) && (i == 0 || s[i] != s[i - 1]);
      unsigned mask = __ballot_sync(0xffffffffu, keep);
      if (pass == 1 && keep) colidx[base + out + __popc(mask & ((1u << lane) - 1))] = s[i];
      out += __popc(mask);
    }
    if (pass == 0 && lane == 0) rowcnt[v] = out;
    __syncwarp();
  }
}

// Thread per (e, i): binary search each ep[e, j] in row ep[e, i].
__global__ void slots_build(const int32_t *ep, int64_t nE, int32_t card, int32_t n,
                           const uint32_t *rowptr, const uint32_t *colidx,
                           uint32_t *slots, int *err) {
  const int64_t m = nE * card;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < m;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / card;
    const int32_t row = ep[t];
    if (row < 0 || row >= n) {
      dev_fail(err, DEV_BAD_ENDPOINT);
      for (int j = 0; j < card; ++j) slots[t * card + j] = 0xffffffffu;
      continue;
    }
    const uint32_t lo0 = rowptr[row], hi0 = rowptr[row + 1];
    for (int j = 0; j < card; ++j) {
      const uint32_t col = (uint32_t)ep[e * card + j];
      uint32_t lo = lo0, hi = hi0;
      while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (colidx[mid] < col) lo = mid + 1; else hi = mid;
      }
      if (lo >= hi0 || colidx[lo] != col) {
        dev_fail(err, DEV_SLOT_MISSING);
        lo = 0xffffffffu;
      }
      slots[t * card + j] = lo;
    }
  }
}

// Shared-memory capacity (keys per warp) for a maximum list length.
static int sort_cap(uint32_t maxlen) {
  int p = 32;
  while ((uint32_t)p < maxlen) p <<= 1;
  return p;
}

static int max_row_len(Ctx *c, Scratch &s, const uint32_t *ptr, int32_t n,
                       uint32_t *h_max) {
  uint32_t *d = s.alloc<uint32_t>(1);
  SG_CHECK_CUDA(cudaMemsetAsync(d, 0, 4, c->stream));
  max_u32_diff<<<grid_for(c, n, 256, 4), 256, 0, c->stream>>>(ptr, n, d);
  SG_CHECK_LAUNCH();
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, d, 4, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  *h_max = *(uint32_t *)c->h_stage;
  return SG_OK;
}

// Warps per block so that cap keys per warp fit the shared-memory budget.
static int warps_for_cap(int cap) {
  const int budget = 96 * 1024;
  int w = budget / (cap * 4);
  if (w > 8) w = 8;
  return w;
}

constexpr int MAX_SORT_CAP = 16384;  // keys per warp (64 KB)

static int check_pattern_args(int32_t n, const int32_t *ep, int64_t nE, int32_t card) {
  SG_REQUIRE(n >= 0 && nE >= 0 && card >= 1 && card <= 64,
             "pattern: bad sizes n=%d nE=%lld card=%d", n, (long long)nE, card);
  SG_REQUIRE(nE == 0 || ep, "pattern: endpoints is null");
  SG_REQUIRE(nE * (int64_t)card < (int64_t)0xffffffffll,
             "pattern: nE*card must fit in uint32");
  return SG_OK;
}

}  // namespace sg

using namespace sg;

extern "C" {

int sg_incidence_build(sg_ctx *h, int32_t n, const int32_t *ep, int64_t nE,
                       int32_t card, uint32_t *ve_ptr, uint32_t *ve_idx) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && ve_ptr && (nE == 0 || ve_idx), "sg_incidence_build: null argument");
  SG_TRY(check_pattern_args(n, ep, nE, card));
  const int64_t m = nE * card;
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(n + 1, 4) * 2 + scan_scratch_bytes(n) + 512));
  uint32_t *cnt = s.alloc<uint32_t>(n + 1);
  uint32_t *cursor = s.alloc<uint32_t>(n + 1);
  SG_CHECK_CUDA(cudaMemsetAsync(cnt, 0, (n + 1) * sizeof(uint32_t), c->stream));
  if (m > 0) {
    inc_count<<<grid_for(c, m, 256, 8), 256, 0, c->stream>>>(ep, m, n, cnt, c->d_err);
    SG_CHECK_LAUNCH();
  }
  SG_TRY(exclusive_scan_u32(c, s, cnt, ve_ptr, n));
  SG_TRY(check_device_error(c, "sg_incidence_build"));
  if (m == 0) return SG_OK;
  SG_CHECK_CUDA(cudaMemcpyAsync(cursor, ve_ptr, n * sizeof(uint32_t),
                                cudaMemcpyDeviceToDevice, c->stream));
  inc_fill<<<grid_for(c, m, 256, 8), 256, 0, c->stream>>>(ep, m, n, cursor, ve_idx);
  SG_CHECK_LAUNCH();
  uint32_t maxdeg = 0;
  SG_TRY(max_row_len(c, s, ve_ptr, n, &maxdeg));
  if (maxdeg > (uint32_t)MAX_SORT_CAP)
    return set_error(SG_ERR_UNSUPPORTED,
                     "sg_incidence_build: vertex degree %u exceeds %d", maxdeg, MAX_SORT_CAP);
  const int cap = sort_cap(maxdeg);
  const int w = warps_for_cap(cap);
  if ((size_t)w * cap * 4 > 48 * 1024)
    SG_CHECK_CUDA(cudaFuncSetAttribute(inc_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       w * cap * 4));
  inc_sort<<<grid_for(c, (int64_t)n * 32, w * 32, 8), w * 32, (size_t)w * cap * 4, c->stream>>>(
      ve_ptr, ve_idx, n, cap, c->d_err);
  SG_CHECK_LAUNCH();
  return check_device_error(c, "sg_incidence_build");
}

static int rows_launch(Ctx *c, Scratch &s, const int32_t *ep, int32_t card,
                       const uint32_t *ve_ptr, const uint32_t *ve_idx, int32_t n,
                       int pass, uint32_t *rowcnt, const uint32_t *rowptr,
                       uint32_t *colidx) {
  uint32_t maxdeg = 0;
  SG_TRY(max_row_len(c, s, ve_ptr, n, &maxdeg));
  const uint64_t maxlen = (uint64_t)maxdeg * card;
  if (maxlen > (uint64_t)MAX_SORT_CAP)
    return set_error(SG_ERR_UNSUPPORTED,
                     "sg_pattern: %llu candidate columns in one row exceed %d",
                     (unsigned long long)maxlen, MAX_SORT_CAP);
  const int cap = sort_cap((uint32_t)maxlen);
  const int w = warps_for_cap(cap);
  const size_t sh = (size_t)w * cap * 4;
  if (sh > 48 * 1024)
    SG_CHECK_CUDA(cudaFuncSetAttribute(rows_build,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  rows_build<<<grid_for(c, (int64_t)n * 32, w * 32, 8), w * 32, sh, c->stream>>>(
      ep, card, ve_ptr, ve_idx, n, cap, pass, rowcnt, rowptr, colidx, c->d_err);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

int sg_pattern_count(sg_ctx *h, int32_t n, const int32_t *ep, int64_t nE,
                     int32_t card, const uint32_t *ve_ptr, const uint32_t *ve_idx,
                     uint32_t *rowptr, int64_t *h_nnzb) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && ve_ptr && rowptr && h_nnzb, "sg_pattern_count: null argument");
  SG_TRY(check_pattern_args(n, ep, nE, card));
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(n + 1, 4) + scan_scratch_bytes(n) + 1024));
  uint32_t *rowcnt = s.alloc<uint32_t>(n + 1);
  SG_TRY(rows_launch(c, s, ep, card, ve_ptr, ve_idx, n, 0, rowcnt, nullptr, nullptr));
  SG_TRY(exclusive_scan_u32(c, s, rowcnt, rowptr, n));
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, rowptr + n, 4, cudaMemcpyDeviceToHost, c->stream));
  SG_TRY(check_device_error(c, "sg_pattern_count"));
  *h_nnzb = *(uint32_t *)c->h_stage;
  return SG_OK;
}

int sg_pattern_fill(sg_ctx *h, int32_t n, const int32_t *ep, int64_t nE,
                    int32_t card, const uint32_t *ve_ptr, const uint32_t *ve_idx,
                    const uint32_t *rowptr, uint32_t *colidx) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && ve_ptr && rowptr && (nE == 0 || colidx), "sg_pattern_fill: null argument");
  SG_TRY(check_pattern_args(n, ep, nE, card));
  Scratch s(c);
  SG_TRY(s.reserve(1024));
  SG_TRY(rows_launch(c, s, ep, card, ve_ptr, ve_idx, n, 1, nullptr, rowptr, colidx));
  return check_device_error(c, "sg_pattern_fill");
}

int sg_slots_build(sg_ctx *h, int32_t n, const int32_t *ep, int64_t nE,
                   int32_t card, const uint32_t *rowptr, const uint32_t *colidx,
                   uint32_t *slots) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && rowptr && (nE == 0 || (colidx && slots)), "sg_slots_build: null argument");
  SG_TRY(check_pattern_args(n, ep, nE, card));
  const int64_t m = nE * card;
  if (m == 0) return SG_OK;
  slots_build<<<grid_for(c, m, 256, 8), 256, 0, c->stream>>>(ep, nE, card, n, rowptr,
                                                              colidx, slots, c->d_err);
  SG_CHECK_LAUNCH();
  return check_device_error(c, "sg_slots_build");
}

}  // extern "C"
