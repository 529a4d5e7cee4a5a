// Blocked-CSR SpMV device code, shared by sg_bspmv and the CG kernels.
//
// Layout (the reference's Indexed storage, src/lower/lower_accesses.cpp:
// 120-245): rowptr[n+1], colidx[nnzb] (sorted), vals[nnzb*bs*bs] with each
// block row-major.
//
// Work split: a group of G lanes owns one block row; lane k of the group
// takes blocks rowptr[r]+k, +G, ...  For bs = 3 each lane streams its block's
// 9 values (consecutive lanes -> consecutive 36-byte blocks, so a group's
// loads cover whole cache lines), gathers x[c*3 .. c*3+2], and keeps three
// partial sums; the group then reduces them with xor-shuffles.  This is the
// lowered loop nest's arithmetic (row-of-block dot over the block columns,
// summed over the row's blocks) with the block sum split across G lanes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

template <typename T> __device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

// Streaming load: matrix values are read once per SpMV; keep them out of L1.
__device__ __forceinline__ float ld_stream(const float *p) {
  float v;
  asm volatile("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_stream(const double *p) {
  double v;
  asm volatile("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

template <int G> __device__ __forceinline__ unsigned group_mask() {
  if (G == 32) return 0xffffffffu;
  const unsigned lane = threadIdx.x & 31;
  return ((1u << G) - 1u) << (lane & ~(unsigned)(G - 1));
}

template <int G, typename AT>
__device__ __forceinline__ AT group_sum(AT v, unsigned mask) {
#pragma unroll
  for (int o = G >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
  return v;
}

// y_row (3 components) = sum over the row's 3x3 blocks of A_blk * x_col.
// Every lane of the group returns the full sums.
template <int G, typename VT, typename XT, typename AT>
__device__ __forceinline__ void bsr3_row(const uint32_t *__restrict__ rowptr,
                                         const uint32_t *__restrict__ colidx,
                                         const VT *__restrict__ vals,
                                         const XT *__restrict__ x, int64_t row,
                                         int gl, unsigned mask, AT &y0, AT &y1,
                                         AT &y2) {
  const uint32_t e = ldg(rowptr + row + 1);
  uint32_t b = ldg(rowptr + row) + gl;
  AT a0 = 0, a1 = 0, a2 = 0;
#pragma unroll 2
  for (; b < e; b += G) {
    const uint32_t c = ldg(colidx + b);
    const VT *v = vals + (size_t)b * 9;
    const AT x0 = (AT)ldg(x + (size_t)c * 3 + 0);
    const AT x1 = (AT)ldg(x + (size_t)c * 3 + 1);
    const AT x2 = (AT)ldg(x + (size_t)c * 3 + 2);
    const AT v0 = (AT)ld_stream(v + 0), v1 = (AT)ld_stream(v + 1), v2 = (AT)ld_stream(v + 2);
    const AT v3 = (AT)ld_stream(v + 3), v4 = (AT)ld_stream(v + 4), v5 = (AT)ld_stream(v + 5);
    const AT v6 = (AT)ld_stream(v + 6), v7 = (AT)ld_stream(v + 7), v8 = (AT)ld_stream(v + 8);
    a0 += v0 * x0 + v1 * x1 + v2 * x2;
    a1 += v3 * x0 + v4 * x1 + v5 * x2;
    a2 += v6 * x0 + v7 * x1 + v8 * x2;
  }
  y0 = group_sum<G>(a0, mask);
  y1 = group_sum<G>(a1, mask);
  y2 = group_sum<G>(a2, mask);
}

// Scalar CSR row (bs = 1).
template <int G, typename VT, typename XT, typename AT>
__device__ __forceinline__ AT csr_row(const uint32_t *__restrict__ rowptr,
                                      const uint32_t *__restrict__ colidx,
                                      const VT *__restrict__ vals,
                                      const XT *__restrict__ x, int64_t row,
                                      int gl, unsigned mask) {
  const uint32_t e = ldg(rowptr + row + 1);
  uint32_t b = ldg(rowptr + row) + gl;
  AT a = 0;
#pragma unroll 4
  for (; b < e; b += G) a += (AT)ld_stream(vals + b) * (AT)ldg(x + ldg(colidx + b));
  return group_sum<G>(a, mask);
}

// Generic bs: the group's lanes split the row's blocks; out[bs] per lane.
template <int G, int BS, typename VT, typename XT, typename AT>
__device__ __forceinline__ void bsr_row(const uint32_t *__restrict__ rowptr,
                                        const uint32_t *__restrict__ colidx,
                                        const VT *__restrict__ vals,
                                        const XT *__restrict__ x, int64_t row,
                                        int gl, unsigned mask, AT *out) {
  const uint32_t e = ldg(rowptr + row + 1);
  AT a[BS];
#pragma unroll
  for (int i = 0; i < BS; ++i) a[i] = 0;
  for (uint32_t b = ldg(rowptr + row) + gl; b < e; b += G) {
    const uint32_t c = ldg(colidx + b);
    const VT *v = vals + (size_t)b * BS * BS;
#pragma unroll
    for (int i = 0; i < BS; ++i) {
      AT t = 0;
#pragma unroll
      for (int j = 0; j < BS; ++j) t += (AT)ld_stream(v + i * BS + j) * (AT)ldg(x + (size_t)c * BS + j);
      a[i] += t;
    }
  }
#pragma unroll
  for (int i = 0; i < BS; ++i) out[i] = group_sum<G>(a[i], mask);
}

}  // namespace sg
