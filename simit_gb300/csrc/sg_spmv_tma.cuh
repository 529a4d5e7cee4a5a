// TMA-staged 3x3 blocked SpMV.
//
// A CTA walks tiles of ROWS consecutive block rows (persistent grid).  A
// tile's values and column indices are contiguous in the CSR arrays, so one
// thread issues two 1-D bulk copies (cp.async.bulk, 16-byte aligned head,
// the unaligned tail of at most 15 bytes loaded by threads) into one of two
// shared-memory buffers while the CTA computes the previous tile from the
// other.  HBM therefore sees full-line streaming reads of the matrix, and the
// compute side reads each block's 9 values from shared memory (lane stride 9
// words: bank-conflict free).  x is gathered through L1/L2; y is written by
// the group's lanes.  With DOT the kernel also returns the CTA's partial of
// p.q (the CG K1 epilogue).
#pragma once
#include "sg_solver_kernels.cuh"
#include "sg_tma.cuh"

namespace sg {

template <typename MT>
__host__ __device__ inline size_t tma_vbytes(int capb) {
  return (((size_t)capb * 9 * sizeof(MT) + 32) + 15) & ~size_t(15);
}
__host__ __device__ inline size_t tma_cbytes(int capb) {
  return (((size_t)capb * 4 + 32) + 15) & ~size_t(15);
}
template <typename MT> inline size_t tma_smem_bytes(int capb, int nst) {
  return 64 + (size_t)nst * (tma_vbytes<MT>(capb) + tma_cbytes(capb));
}

// NST-stage pipeline: while the CTA computes tile k, the copies of tiles
// k+1 .. k+NST-1 are in flight.
template <int G, int ROWS, int NST, typename MT, typename VT, bool DOT>
__global__ void __launch_bounds__(ROWS *G)
    k_bsr3_tma(const SolveCtl *__restrict__ ctl, int32_t n, const uint32_t *__restrict__ rowptr,
               const uint32_t *__restrict__ colidx, const MT *__restrict__ vals,
               const VT *__restrict__ x, VT *__restrict__ y, double *__restrict__ part, int capb,
               int *err) {
  static_assert(NST >= 2 && NST <= 6, "stages");
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double shred[33];
  __shared__ int ok_flag;
  if (ctl && ctl->status != ST_RUNNING) return;
  const size_t vbytes = tma_vbytes<MT>(capb), cbytes = tma_cbytes(capb);
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm);
  unsigned char *base = sm + 64;
  auto vbuf = [&](int b) { return reinterpret_cast<MT *>(base + (size_t)b * (vbytes + cbytes)); };
  auto cbuf = [&](int b) {
    return reinterpret_cast<uint32_t *>(base + (size_t)b * (vbytes + cbytes) + vbytes);
  };
  const int ntiles = (n + ROWS - 1) / ROWS;
  constexpr size_t S = sizeof(MT);
  if (threadIdx.x == 0) {
    for (int b = 0; b < NST; ++b) mbar_init(&bar[b], 1);
    mbar_fence_init();
  }
  __syncthreads();

  auto tile_range = [&](int tile, uint32_t &b0, uint32_t &b1) {
    const int r0 = tile * ROWS;
    const int r1 = min(n, r0 + ROWS);
    b0 = rowptr[r0];
    b1 = rowptr[r1];
  };
  auto issue = [&](int tile, int b) {
    uint32_t b0, b1;
    tile_range(tile, b0, b1);
    const size_t vs = ((size_t)b0 * 9 * S) & ~size_t(15), ve = ((size_t)b1 * 9 * S) & ~size_t(15);
    const size_t cs = ((size_t)b0 * 4) & ~size_t(15), ce = ((size_t)b1 * 4) & ~size_t(15);
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bar[b], (uint32_t)((ve - vs) + (ce - cs)));
    if (ve > vs)
      bulk_g2s(vbuf(b), reinterpret_cast<const unsigned char *>(vals) + vs, (uint32_t)(ve - vs),
               &bar[b]);
    if (ce > cs)
      bulk_g2s(cbuf(b), reinterpret_cast<const unsigned char *>(colidx) + cs,
               (uint32_t)(ce - cs), &bar[b]);
  };

  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = group_mask<G>();
  double acc = 0;
  // local tile k of this CTA is global tile blockIdx.x + k*gridDim.x
  const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  if (threadIdx.x == 0)
    for (int k = 0; k < NST - 1 && k < my_tiles; ++k) issue(blockIdx.x + k * gridDim.x, k);
  for (int k = 0; k < my_tiles; ++k) {
    const int b = k % NST;
    const int tile = blockIdx.x + k * gridDim.x;
    if (threadIdx.x == 0) {
      const int kn = k + NST - 1;
      if (kn < my_tiles) issue(blockIdx.x + kn * gridDim.x, kn % NST);
      const bool ok = mbar_wait(&bar[b], (uint32_t)((k / NST) & 1));
      ok_flag = ok ? 1 : 0;
      if (!ok) {
        atomicCAS(err, 0, 6 /* DEV_TMA_TIMEOUT */);
        // drain the copies still in flight before leaving
        for (int kk = k + 1; kk < my_tiles && kk <= kn; ++kk)
          mbar_wait(&bar[kk % NST], (uint32_t)((kk / NST) & 1));
      }
    }
    __syncthreads();
    if (!ok_flag) break;
    MT *vb = vbuf(b);
    uint32_t *cb = cbuf(b);
    uint32_t b0, b1;
    tile_range(tile, b0, b1);
    const size_t vs = ((size_t)b0 * 9 * S) & ~size_t(15), ve = ((size_t)b1 * 9 * S) & ~size_t(15);
    const size_t cs = ((size_t)b0 * 4) & ~size_t(15), ce = ((size_t)b1 * 4) & ~size_t(15);
    // unaligned tails (< 16 bytes each)
    const int vt = (int)(((size_t)b1 * 9 * S - ve) / S);
    const int ct = (int)(((size_t)b1 * 4 - ce) / 4);
    if ((int)threadIdx.x < vt) vb[(ve - vs) / S + threadIdx.x] = vals[ve / S + threadIdx.x];
    if ((int)threadIdx.x >= 32 && (int)threadIdx.x < 32 + ct)
      cb[(ce - cs) / 4 + threadIdx.x - 32] = colidx[ce / 4 + threadIdx.x - 32];
    __syncthreads();
    const int r = tile * ROWS + (int)(threadIdx.x / G);
    if (r < n) {
      const uint32_t e = rowptr[r + 1];
      VT a0 = 0, a1 = 0, a2 = 0;
      const size_t voff = vs / S, coff = cs / 4;
#pragma unroll 4
      for (uint32_t q = rowptr[r] + gl; q < e; q += G) {
        const uint32_t c = cb[q - coff];
        const MT *v = vb + ((size_t)q * 9 - voff);
        const VT x0 = ldg(x + (size_t)c * 3 + 0), x1 = ldg(x + (size_t)c * 3 + 1),
                 x2 = ldg(x + (size_t)c * 3 + 2);
        a0 += (VT)v[0] * x0 + (VT)v[1] * x1 + (VT)v[2] * x2;
        a1 += (VT)v[3] * x0 + (VT)v[4] * x1 + (VT)v[5] * x2;
        a2 += (VT)v[6] * x0 + (VT)v[7] * x1 + (VT)v[8] * x2;
      }
      a0 = group_sum<G>(a0, mask);
      a1 = group_sum<G>(a1, mask);
      a2 = group_sum<G>(a2, mask);
      if (gl < 3) {
        const VT yv = gl == 0 ? a0 : (gl == 1 ? a1 : a2);
        y[(size_t)r * 3 + gl] = yv;
        if (DOT) acc += (double)x[(size_t)r * 3 + gl] * (double)yv;
      }
    }
    __syncthreads();
  }
  if (DOT) {
    const double t = block_sum(acc, shred);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

}  // namespace sg
