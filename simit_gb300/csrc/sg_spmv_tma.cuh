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

template <typename MT, int BB = 9>
__host__ __device__ inline size_t tma_vbytes(int capb) {
  return (((size_t)capb * BB * sizeof(MT) + 32) + 15) & ~size_t(15);
}
__host__ __device__ inline size_t tma_cbytes(int capb) {
  return (((size_t)capb * 4 + 32) + 15) & ~size_t(15);
}
template <typename MT> inline size_t tma_smem_bytes(int capb, int nst) {
  return 64 + (size_t)nst * (tma_vbytes<MT>(capb) + tma_cbytes(capb));
}

// y_r = (A x)_r for block row r from its tile's values vb and columns cb
// (block q at vb[q*9 - voff], cb[q - coff]); G lanes per row, lane gl takes
// blocks rowptr[r]+gl, +G, ...  The first U blocks of each lane (rows of up
// to 24 blocks) use a fixed, predicated trip count so all of the lane's x
// gathers are in flight at once; the remainder loop keeps the same
// accumulation order.  With DOT, acc accumulates x_r . y_r (DotAcc).
template <int G, typename MT, typename VT, bool DOT>
__device__ __forceinline__ void tile_row(int64_t r, int gl, unsigned mask,
                                         const uint32_t *__restrict__ rowptr,
                                         const MT *__restrict__ vb,
                                         const uint32_t *__restrict__ cb, size_t voff,
                                         size_t coff, const VT *__restrict__ x,
                                         VT *__restrict__ y, DotAcc<VT> &acc) {
  const uint32_t e = rowptr[r + 1];
  VT a0 = 0, a1 = 0, a2 = 0;
  constexpr int U = (24 + G - 1) / G;
  const uint32_t q0 = rowptr[r] + gl;
  VT xg[U][3];
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const uint32_t q = q0 + k * G;
    if (q < e) {
      const uint32_t c = cb[q - coff];
      xg[k][0] = ldg(x + (size_t)c * 3 + 0);
      xg[k][1] = ldg(x + (size_t)c * 3 + 1);
      xg[k][2] = ldg(x + (size_t)c * 3 + 2);
    }
  }
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const uint32_t q = q0 + k * G;
    if (q < e) {
      const MT *v = vb + ((size_t)q * 9 - voff);
      const VT x0 = xg[k][0], x1 = xg[k][1], x2 = xg[k][2];
      a0 += (VT)v[0] * x0 + (VT)v[1] * x1 + (VT)v[2] * x2;
      a1 += (VT)v[3] * x0 + (VT)v[4] * x1 + (VT)v[5] * x2;
      a2 += (VT)v[6] * x0 + (VT)v[7] * x1 + (VT)v[8] * x2;
    }
  }
#pragma unroll 4
  for (uint32_t q = q0 + U * G; q < e; q += G) {
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
  if (G >= 3) {
    if (gl < 3) {
      const VT yv = gl == 0 ? a0 : (gl == 1 ? a1 : a2);
      y[(size_t)r * 3 + gl] = yv;
      if (DOT) acc.add(x[(size_t)r * 3 + gl], yv);
    }
  } else if (gl == 0) {  // fewer than 3 lanes: lane 0 writes the row
    y[(size_t)r * 3 + 0] = a0;
    y[(size_t)r * 3 + 1] = a1;
    y[(size_t)r * 3 + 2] = a2;
    if (DOT) {
      acc.add(x[(size_t)r * 3], a0);
      acc.add(x[(size_t)r * 3 + 1], a1);
      acc.add(x[(size_t)r * 3 + 2], a2);
    }
  }
}

// Scalar CSR row (1x1 blocks): y_r = sum_q vb[q - voff] x[cb[q - coff]],
// same lane split, predicated gathers and accumulation order as tile_row.
template <int G, typename MT, typename VT, bool DOT>
__device__ __forceinline__ void tile_row1(int64_t r, int gl, unsigned mask,
                                          const uint32_t *__restrict__ rowptr,
                                          const MT *__restrict__ vb,
                                          const uint32_t *__restrict__ cb, size_t voff,
                                          size_t coff, const VT *__restrict__ x,
                                          VT *__restrict__ y, DotAcc<VT> &acc) {
  const uint32_t e = rowptr[r + 1];
  VT a = 0;
  constexpr int U = (24 + G - 1) / G;
  const uint32_t q0 = rowptr[r] + gl;
  VT xg[U];
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const uint32_t q = q0 + k * G;
    if (q < e) xg[k] = ldg(x + cb[q - coff]);
  }
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const uint32_t q = q0 + k * G;
    if (q < e) a += (VT)vb[q - voff] * xg[k];
  }
#pragma unroll 4
  for (uint32_t q = q0 + U * G; q < e; q += G) a += (VT)vb[q - voff] * ldg(x + cb[q - coff]);
  a = group_sum<G>(a, mask);
  if (gl == 0) {
    y[r] = a;
    if (DOT) acc.add(x[r], a);
  }
}

// NST-stage pipeline: while the CTA computes tile k, the copies of tiles
// k+1 .. k+NST-1 are in flight.  A tile of more than capb blocks (the
// buffers' capacity) is never staged: it is read straight from global
// memory, so a stale tile statistic costs speed, never memory safety.
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
    if (b1 - b0 > (uint32_t)capb) {  // larger than the buffers: read from global
      mbar_arrive_expect_tx(&bar[b], 0);
      return;
    }
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
  DotAcc<VT> acc;
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
        // no new copies; wait (bounded) on every barrier with a copy still
        // in flight, this tile's included, before leaving; if one of those
        // waits runs out too, a copy may still land in shared memory after
        // the CTA exits: record that (the results are then undefined and
        // the context should be reset)
        bool drained = true;
        for (int kk = k; kk < my_tiles && kk <= kn; ++kk)
          drained = mbar_wait(&bar[kk % NST], (uint32_t)((kk / NST) & 1)) && drained;
        if (!drained) atomicExch(err, 8 /* DEV_TMA_UNDRAINED */);
      }
    }
    __syncthreads();
    if (!ok_flag) break;
    uint32_t b0, b1;
    tile_range(tile, b0, b1);
    const bool staged = b1 - b0 <= (uint32_t)capb;
    const size_t vs = staged ? ((size_t)b0 * 9 * S) & ~size_t(15) : 0;
    const size_t cs = staged ? ((size_t)b0 * 4) & ~size_t(15) : 0;
    if (staged) {
      // unaligned tails (< 16 bytes each)
      const size_t ve = ((size_t)b1 * 9 * S) & ~size_t(15), ce = ((size_t)b1 * 4) & ~size_t(15);
      const int vt = (int)(((size_t)b1 * 9 * S - ve) / S);
      const int ct = (int)(((size_t)b1 * 4 - ce) / 4);
      if ((int)threadIdx.x < vt) vbuf(b)[(ve - vs) / S + threadIdx.x] = vals[ve / S + threadIdx.x];
      if ((int)threadIdx.x >= 32 && (int)threadIdx.x < 32 + ct)
        cbuf(b)[(ce - cs) / 4 + threadIdx.x - 32] = colidx[ce / 4 + threadIdx.x - 32];
    }
    __syncthreads();
    const int r = tile * ROWS + (int)(threadIdx.x / G);
    if (r < n) {
      // two inlined copies: shared-memory loads for a staged tile, global
      // loads for an oversize one
      if (staged)
        tile_row<G, MT, VT, DOT>(r, gl, mask, rowptr, vbuf(b), cbuf(b), vs / S, cs / 4, x, y, acc);
      else
        tile_row<G, MT, VT, DOT>(r, gl, mask, rowptr, vals, colidx, 0, 0, x, y, acc);
    }
    __syncthreads();
  }
  if (DOT) {  // CG K1: the last CTA leaves the p.q total in ctl->pq_tot
    const double t = block_sum(acc.value(), shred);
    SolveCtl *c = const_cast<SolveCtl *>(ctl);
    finalize_partials(&t, 1, part, &c->tick1, &c->pq_tot, shred);
  }
}

}  // namespace sg

namespace sg {

// Per-warp variant: every warp runs its own NST-stage bulk-copy pipeline
// over tiles of RW = 32/G consecutive block rows (global warp w takes tiles
// w, w + total warps, ...), waits on its own mbarriers and synchronises only
// with __syncwarp, so no warp waits for another's copy or compute.  Each
// warp's buffers hold capb blocks; a larger tile (the caller's statistics
// were stale, or a very long row) is read straight from global memory.
constexpr int WTMA_WARPS = 4;

template <typename MT, int BB = 9> inline size_t wtma_smem_bytes(int capb, int nst) {
  return (((size_t)WTMA_WARPS * nst * 8 + 15) & ~size_t(15)) +
         (size_t)WTMA_WARPS * nst * (tma_vbytes<MT, BB>(capb) + tma_cbytes(capb));
}

// Body shared by the 3x3 (BS = 3) and scalar CSR (BS = 1) kernels.  A warp
// tile is P passes of 32/G rows (P > 1 makes the bulk copies of short
// scalar rows larger).
template <int BS, int G, int NST, int P, typename MT, typename VT, bool DOT>
__device__ __forceinline__ void wtma_body(const SolveCtl *__restrict__ ctl, int32_t n,
                                          const uint32_t *__restrict__ rowptr,
                                          const uint32_t *__restrict__ colidx,
                                          const MT *__restrict__ vals, const VT *__restrict__ x,
                                          VT *__restrict__ y, double *__restrict__ part,
                                          int capb, int *err, unsigned char *sm,
                                          double *shred) {
  static_assert(NST >= 2 && NST <= 6, "stages");
  static_assert(BS == 1 || BS == 3, "block size");
  constexpr int RW = 32 / G * P;
  constexpr int BB = BS * BS;
  constexpr size_t S = sizeof(MT);
  pdl_wait_and_release();
  if (ctl && ctl->status != ST_RUNNING) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t vbytes = tma_vbytes<MT, BB>(capb), cbytes = tma_cbytes(capb);
  const size_t stage = vbytes + cbytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm) + warp * NST;
  unsigned char *base =
      sm + (((size_t)WTMA_WARPS * NST * 8 + 15) & ~size_t(15)) + (size_t)warp * NST * stage;
  auto vbuf = [&](int b) { return reinterpret_cast<MT *>(base + (size_t)b * stage); };
  auto cbuf = [&](int b) { return reinterpret_cast<uint32_t *>(base + (size_t)b * stage + vbytes); };
  if (lane == 0) {
    for (int b = 0; b < NST; ++b) mbar_init(&bar[b], 1);
    mbar_fence_init();
  }
  __syncwarp();
  const int64_t ntiles = ((int64_t)n + RW - 1) / RW;
  const int64_t gw = (int64_t)blockIdx.x * WTMA_WARPS + warp;
  const int64_t nw = (int64_t)gridDim.x * WTMA_WARPS;
  const int64_t my = gw < ntiles ? (ntiles - 1 - gw) / nw + 1 : 0;
  auto issue = [&](int64_t tile, int b) {
    const int64_t r0 = tile * RW;
    const int64_t r1 = min((int64_t)n, r0 + RW);
    const uint32_t b0 = rowptr[r0], b1 = rowptr[r1];
    const size_t vs = ((size_t)b0 * BB * S) & ~size_t(15), ve = ((size_t)b1 * BB * S) & ~size_t(15);
    const size_t cs = ((size_t)b0 * 4) & ~size_t(15), ce = ((size_t)b1 * 4) & ~size_t(15);
    fence_proxy_async_smem();
    if (b1 - b0 > (uint32_t)capb) {  // larger than the buffers: read from global
      mbar_arrive_expect_tx(&bar[b], 0);
      return;
    }
    mbar_arrive_expect_tx(&bar[b], (uint32_t)((ve - vs) + (ce - cs)));
    if (ve > vs)
      bulk_g2s(vbuf(b), reinterpret_cast<const unsigned char *>(vals) + vs, (uint32_t)(ve - vs),
               &bar[b]);
    if (ce > cs)
      bulk_g2s(cbuf(b), reinterpret_cast<const unsigned char *>(colidx) + cs,
               (uint32_t)(ce - cs), &bar[b]);
  };
  if (lane == 0)
    for (int k = 0; k < NST - 1 && k < my; ++k) issue(gw + k * nw, k);
  const int gl = lane & (G - 1);
  const unsigned mask = group_mask<G>();
  DotAcc<VT> acc;
  for (int64_t k = 0; k < my; ++k) {
    const int b = (int)(k % NST);
    const int64_t tile = gw + k * nw;
    const int64_t kn = k + NST - 1;
    if (lane == 0 && kn < my) issue(gw + kn * nw, (int)(kn % NST));
    const bool ok = __all_sync(0xffffffffu, mbar_wait(&bar[b], (uint32_t)((k / NST) & 1)));
    if (!ok) {
      if (lane == 0) {
        atomicCAS(err, 0, 6 /* DEV_TMA_TIMEOUT */);
        // drain every barrier with a copy in flight (see k_bsr3_tma)
        bool drained = true;
        for (int64_t kk = k; kk < my && kk <= kn; ++kk)
          drained = mbar_wait(&bar[kk % NST], (uint32_t)((kk / NST) & 1)) && drained;
        if (!drained) atomicExch(err, 8 /* DEV_TMA_UNDRAINED */);
      }
      break;
    }
    const int64_t r0 = tile * RW;
    const uint32_t b0 = rowptr[r0], b1 = rowptr[min((int64_t)n, r0 + RW)];
    const bool staged = b1 - b0 <= (uint32_t)capb;
    const size_t vs = staged ? ((size_t)b0 * BB * S) & ~size_t(15) : 0;
    const size_t cs = staged ? ((size_t)b0 * 4) & ~size_t(15) : 0;
    if (staged) {
      // unaligned tails (< 16 bytes each)
      const size_t ve = ((size_t)b1 * BB * S) & ~size_t(15), ce = ((size_t)b1 * 4) & ~size_t(15);
      const int vt = (int)(((size_t)b1 * BB * S - ve) / S);
      const int ct = (int)(((size_t)b1 * 4 - ce) / 4);
      if (lane < vt) vbuf(b)[(ve - vs) / S + lane] = vals[ve / S + lane];
      if (lane >= 16 && lane < 16 + ct)
        cbuf(b)[(ce - cs) / 4 + lane - 16] = colidx[ce / 4 + lane - 16];
    }
    __syncwarp();
#pragma unroll
    for (int pp = 0; pp < P; ++pp) {
    const int64_t r = r0 + pp * (32 / G) + lane / G;
    if (r < n) {
      if (BS == 3) {
        if (staged)
          tile_row<G, MT, VT, DOT>(r, gl, mask, rowptr, vbuf(b), cbuf(b), vs / S, cs / 4, x, y,
                                   acc);
        else
          tile_row<G, MT, VT, DOT>(r, gl, mask, rowptr, vals, colidx, 0, 0, x, y, acc);
      } else {
        if (staged)
          tile_row1<G, MT, VT, DOT>(r, gl, mask, rowptr, vbuf(b), cbuf(b), vs / S, cs / 4, x, y,
                                    acc);
        else
          tile_row1<G, MT, VT, DOT>(r, gl, mask, rowptr, vals, colidx, 0, 0, x, y, acc);
      }
    }
    }
    __syncwarp();
  }
  if (DOT) {  // CG K1: the last CTA leaves the p.q total in ctl->pq_tot
    const double t = block_sum(acc.value(), shred);
    SolveCtl *c = const_cast<SolveCtl *>(ctl);
    finalize_partials(&t, 1, part, &c->tick1, &c->pq_tot, shred);
  }
}

template <int G, int NST, typename MT, typename VT, bool DOT>
__global__ void __launch_bounds__(WTMA_WARPS * 32)
    k_bsr3_wtma(const SolveCtl *__restrict__ ctl, int32_t n, const uint32_t *__restrict__ rowptr,
                const uint32_t *__restrict__ colidx, const MT *__restrict__ vals,
                const VT *__restrict__ x, VT *__restrict__ y, double *__restrict__ part,
                int capb, int *err) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double shred[33];
  wtma_body<3, G, NST, 1, MT, VT, DOT>(ctl, n, rowptr, colidx, vals, x, y, part, capb, err, sm,
                                       shred);
}

// Scalar CSR (bs = 1) with the same per-warp pipeline, tiles of P passes.
template <int G, int NST, int P, typename MT, typename VT, bool DOT>
__global__ void __launch_bounds__(WTMA_WARPS * 32)
    k_csr_wtma(const SolveCtl *__restrict__ ctl, int32_t n, const uint32_t *__restrict__ rowptr,
               const uint32_t *__restrict__ colidx, const MT *__restrict__ vals,
               const VT *__restrict__ x, VT *__restrict__ y, double *__restrict__ part,
               int capb, int *err) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double shred[33];
  wtma_body<1, G, NST, P, MT, VT, DOT>(ctl, n, rowptr, colidx, vals, x, y, part, capb, err, sm,
                                       shred);
}

}  // namespace sg
