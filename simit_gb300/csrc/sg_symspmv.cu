// Symmetric-storage 3x3 blocked SpMV (FP32) for matrices whose pattern and
// values are symmetric, as the stiffness matrices of the tet maps are.
//
// Layout.  The upper half (blocks with column >= row) is a CSR of its own:
// urowptr, ucol, uvals (row-major 3x3 blocks).  For every row r the blocks
// below its diagonal are listed in lidx as {c, s}: column c < r and the upper
// slot s of block (c, r), whose transpose block (r, c) is.  Both lists keep
// the full pattern's column order.
//
// Kernel.  The per-warp bulk-copy pipeline of the full-storage kernel, with
// three streams per 8-row warp tile: the tile's upper values, upper columns
// and lower index are copied into shared memory while the warp computes the
// previous tile.  A row's G = 4 lanes take its upper blocks (from shared
// memory) and then its lower blocks, whose values they gather from uvals:
// block (c, r) belongs to a row c < r that an earlier tile streamed, and with
// a locality-preserving vertex order (Morton or Hilbert) about 98 % of such
// rows lie within the last 200K rows, so the re-reads hit L2.  The sum of a
// row is fixed-order: upper blocks, then lower blocks, each lane strided by
// G, then the group reduction.
#include <stdint.h>

#include "sg_internal.cuh"
#include "sg_spmv_tma.cuh"
#include "sg_sym.h"

namespace sg {
namespace {

constexpr int SYM_G = 4;                  // lanes per block row
constexpr int SYM_RW = 32 / SYM_G;        // rows per warp tile
constexpr int SYM_NST_DEFAULT = 3;        // pipeline stages per warp (2..4)

inline __host__ __device__ size_t align16(size_t b) { return (b + 15) & ~size_t(15); }
inline __host__ __device__ size_t sym_vbytes(int capu) { return align16((size_t)capu * 36 + 32); }
inline __host__ __device__ size_t sym_cbytes(int capu) { return align16((size_t)capu * 4 + 32); }
inline __host__ __device__ size_t sym_lbytes(int capl) { return align16((size_t)capl * 8 + 32); }
inline size_t sym_smem_bytes(int capu, int capl, int nst) {
  return align16((size_t)WTMA_WARPS * nst * 8) +
         (size_t)WTMA_WARPS * nst * (sym_vbytes(capu) + sym_cbytes(capu) + sym_lbytes(capl));
}

// First slot of row v (in [s, e)) whose column is >= key.
__device__ __forceinline__ uint32_t lower_bound(const uint32_t *__restrict__ col, uint32_t s,
                                                uint32_t e, uint32_t key) {
  while (s < e) {
    const uint32_t m = s + ((e - s) >> 1);
    if (col[m] < key) s = m + 1;
    else e = m;
  }
  return s;
}

// Per row: the diagonal's slot and the upper / lower block counts.
__global__ void k_sym_count(int32_t n, const uint32_t *__restrict__ rowptr,
                            const uint32_t *__restrict__ colidx, uint32_t *__restrict__ dslot,
                            uint32_t *__restrict__ ucnt, uint32_t *__restrict__ lcnt, int *err) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = rowptr[v], e = rowptr[v + 1];
    uint32_t d = lower_bound(colidx, s, e, (uint32_t)v);
    if (d == e || colidx[d] != (uint32_t)v) {
      atomicCAS(err, 0, (int)DEV_NO_DIAGONAL);
      d = e;  // no upper blocks: keeps every later index in range
    }
    dslot[v] = d;
    ucnt[v] = e - d;
    lcnt[v] = d - s;
  }
}

// Upper columns and the lower index {c, upper slot of (c, v)}.
__global__ void k_sym_pattern(int32_t n, const uint32_t *__restrict__ rowptr,
                              const uint32_t *__restrict__ colidx,
                              const uint32_t *__restrict__ dslot,
                              const uint32_t *__restrict__ urowptr,
                              const uint32_t *__restrict__ lrowptr, uint32_t *__restrict__ ucol,
                              uint2 *__restrict__ lidx, int *err) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t s = rowptr[v], d = dslot[v], e = rowptr[v + 1];
    const uint32_t u0 = urowptr[v], l0 = lrowptr[v];
    for (uint32_t q = d; q < e; ++q) ucol[u0 + (q - d)] = colidx[q];
    for (uint32_t q = s; q < d; ++q) {
      const uint32_t c = colidx[q];
      uint32_t pos = 0;
      if (c < (uint32_t)v) {
        const uint32_t cd = dslot[c], ce = rowptr[c + 1];
        const uint32_t t = lower_bound(colidx, cd, ce, (uint32_t)v);
        if (t < ce && colidx[t] == (uint32_t)v) pos = urowptr[c] + (t - cd);
        else atomicCAS(err, 0, (int)DEV_SLOT_MISSING);  // pattern not symmetric
      } else {
        atomicCAS(err, 0, (int)DEV_SLOT_MISSING);
      }
      lidx[l0 + (q - s)] = make_uint2(c < (uint32_t)n ? c : 0u, pos);
    }
  }
}

// Largest block count of any warp tile of `rows` rows.
__global__ void k_tile_max(int32_t n, const uint32_t *__restrict__ rp, int rows,
                           unsigned *__restrict__ out) {
  unsigned m = 0;
  const int64_t nt = ((int64_t)n + rows - 1) / rows;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r0 = t * rows, r1 = min((int64_t)n, r0 + rows);
    m = max(m, rp[r1] - rp[r0]);
  }
  atomicMax(out, m);
}

// uvals <- the upper blocks of the full values (a warp per row).
__global__ void k_sym_copy(int32_t n, const uint32_t *__restrict__ rowptr,
                           const uint32_t *__restrict__ dslot,
                           const uint32_t *__restrict__ urowptr, const float *__restrict__ vals,
                           float *__restrict__ uvals) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t v = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < n;
       v += warps) {
    const size_t src = (size_t)dslot[v] * 9, dst = (size_t)urowptr[v] * 9;
    const uint32_t len = (rowptr[v + 1] - dslot[v]) * 9;
    for (uint32_t q = lane; q < len; q += 32) uvals[dst + q] = vals[src + q];
  }
}

// y_r for one row: upper blocks (shared memory or global), then lower blocks
// (transposed, values gathered from uvals).  The first U blocks of each lane
// in either half are loaded with fixed, predicated trip counts so their
// gathers are in flight together.
template <bool DOT>
__device__ __forceinline__ void sym_row(int64_t r, int gl, unsigned mask,
                                        const uint32_t *__restrict__ urp,
                                        const uint32_t *__restrict__ lrp,
                                        const float *__restrict__ vb,
                                        const uint32_t *__restrict__ cb,
                                        const uint2 *__restrict__ lb, size_t voff, size_t coff,
                                        size_t loff, uint32_t su0, uint32_t su1,
                                        const float *__restrict__ uv,
                                        const float *__restrict__ x, float *__restrict__ y,
                                        DotAcc<float> &acc) {
  constexpr int G = SYM_G;
  constexpr int U = 2;  // rows of up to 8 upper and 8 lower blocks in one round
  float a0 = 0, a1 = 0, a2 = 0;
  {
    const uint32_t e = urp[r + 1], q0 = urp[r] + gl;
    float xg[U][3];
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
        const float *v = vb + ((size_t)q * 9 - voff);
        a0 += v[0] * xg[k][0] + v[1] * xg[k][1] + v[2] * xg[k][2];
        a1 += v[3] * xg[k][0] + v[4] * xg[k][1] + v[5] * xg[k][2];
        a2 += v[6] * xg[k][0] + v[7] * xg[k][1] + v[8] * xg[k][2];
      }
    }
    for (uint32_t q = q0 + U * G; q < e; q += G) {
      const uint32_t c = cb[q - coff];
      const float *v = vb + ((size_t)q * 9 - voff);
      const float x0 = ldg(x + (size_t)c * 3), x1 = ldg(x + (size_t)c * 3 + 1),
                  x2 = ldg(x + (size_t)c * 3 + 2);
      a0 += v[0] * x0 + v[1] * x1 + v[2] * x2;
      a1 += v[3] * x0 + v[4] * x1 + v[5] * x2;
      a2 += v[6] * x0 + v[7] * x1 + v[8] * x2;
    }
  }
  {
    const uint32_t e = lrp[r + 1], q0 = lrp[r] + gl;
    float lv[U][9], xg[U][3];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const uint32_t q = q0 + k * G;
      if (q < e) {
        const uint2 ent = lb[q - loff];
        // the mirror block is an upper block of this tile: already staged
        const bool in_tile = ent.y >= su0 && ent.y < su1;
        const float *v = in_tile ? vb + ((size_t)ent.y * 9 - voff) : uv + (size_t)ent.y * 9;
#pragma unroll
        for (int w = 0; w < 9; ++w) lv[k][w] = in_tile ? v[w] : ldg(v + w);
        xg[k][0] = ldg(x + (size_t)ent.x * 3 + 0);
        xg[k][1] = ldg(x + (size_t)ent.x * 3 + 1);
        xg[k][2] = ldg(x + (size_t)ent.x * 3 + 2);
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const uint32_t q = q0 + k * G;
      if (q < e) {  // block (r, c) = transpose of the stored (c, r)
        a0 += lv[k][0] * xg[k][0] + lv[k][3] * xg[k][1] + lv[k][6] * xg[k][2];
        a1 += lv[k][1] * xg[k][0] + lv[k][4] * xg[k][1] + lv[k][7] * xg[k][2];
        a2 += lv[k][2] * xg[k][0] + lv[k][5] * xg[k][1] + lv[k][8] * xg[k][2];
      }
    }
    for (uint32_t q = q0 + U * G; q < e; q += G) {
      const uint2 ent = lb[q - loff];
      const float *v = uv + (size_t)ent.y * 9;
      const float x0 = ldg(x + (size_t)ent.x * 3), x1 = ldg(x + (size_t)ent.x * 3 + 1),
                  x2 = ldg(x + (size_t)ent.x * 3 + 2);
      a0 += ldg(v + 0) * x0 + ldg(v + 3) * x1 + ldg(v + 6) * x2;
      a1 += ldg(v + 1) * x0 + ldg(v + 4) * x1 + ldg(v + 7) * x2;
      a2 += ldg(v + 2) * x0 + ldg(v + 5) * x1 + ldg(v + 8) * x2;
    }
  }
  a0 = group_sum<G>(a0, mask);
  a1 = group_sum<G>(a1, mask);
  a2 = group_sum<G>(a2, mask);
  if (gl < 3) {
    const float yv = gl == 0 ? a0 : (gl == 1 ? a1 : a2);
    y[(size_t)r * 3 + gl] = yv;
    if (DOT) acc.add(x[(size_t)r * 3 + gl], yv);
  }
}

template <bool DOT, int NST>
__global__ void __launch_bounds__(WTMA_WARPS * 32, 6)
    k_sbsr3_wtma(const SolveCtl *__restrict__ ctl, int32_t n, const uint32_t *__restrict__ urp,
                 const uint32_t *__restrict__ ucol, const float *__restrict__ uv,
                 const uint32_t *__restrict__ lrp, const uint2 *__restrict__ lidx,
                 const float *__restrict__ x, float *__restrict__ y, double *__restrict__ part,
                 int capu, int capl, int *err) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double shred[33];
  constexpr int RW = SYM_RW, G = SYM_G;
  static_assert(NST >= 2 && NST <= 4, "stages");
  if (ctl && ctl->status != ST_RUNNING) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t vb = sym_vbytes(capu), cbt = sym_cbytes(capu), lbt = sym_lbytes(capl);
  const size_t stage = vb + cbt + lbt;
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm) + warp * NST;
  unsigned char *base = sm + align16((size_t)WTMA_WARPS * NST * 8) + (size_t)warp * NST * stage;
  auto vbuf = [&](int b) { return reinterpret_cast<float *>(base + (size_t)b * stage); };
  auto cbuf = [&](int b) { return reinterpret_cast<uint32_t *>(base + (size_t)b * stage + vb); };
  auto lbuf = [&](int b) {
    return reinterpret_cast<uint2 *>(base + (size_t)b * stage + vb + cbt);
  };
  if (lane == 0) {
    for (int b = 0; b < NST; ++b) mbar_init(&bar[b], 1);
    mbar_fence_init();
  }
  __syncwarp();
  const int64_t ntiles = ((int64_t)n + RW - 1) / RW;
  const int64_t gw = (int64_t)blockIdx.x * WTMA_WARPS + warp;
  const int64_t nw = (int64_t)gridDim.x * WTMA_WARPS;
  const int64_t my = gw < ntiles ? (ntiles - 1 - gw) / nw + 1 : 0;
  auto fits = [&](uint32_t u0, uint32_t u1, uint32_t l0, uint32_t l1) {
    return u1 - u0 <= (uint32_t)capu && l1 - l0 <= (uint32_t)capl;
  };
  auto issue = [&](int64_t tile, int b) {
    const int64_t r0 = tile * RW, r1 = min((int64_t)n, r0 + RW);
    const uint32_t u0 = urp[r0], u1 = urp[r1], l0 = lrp[r0], l1 = lrp[r1];
    fence_proxy_async_smem();
    if (!fits(u0, u1, l0, l1)) {  // larger than the buffers: read from global
      mbar_arrive_expect_tx(&bar[b], 0);
      return;
    }
    const size_t vs = ((size_t)u0 * 36) & ~size_t(15), ve = ((size_t)u1 * 36) & ~size_t(15);
    const size_t cs = ((size_t)u0 * 4) & ~size_t(15), ce = ((size_t)u1 * 4) & ~size_t(15);
    const size_t ls = ((size_t)l0 * 8) & ~size_t(15), le = ((size_t)l1 * 8) & ~size_t(15);
    mbar_arrive_expect_tx(&bar[b], (uint32_t)((ve - vs) + (ce - cs) + (le - ls)));
    if (ve > vs)
      bulk_g2s(vbuf(b), reinterpret_cast<const unsigned char *>(uv) + vs, (uint32_t)(ve - vs),
               &bar[b]);
    if (ce > cs)
      bulk_g2s(cbuf(b), reinterpret_cast<const unsigned char *>(ucol) + cs, (uint32_t)(ce - cs),
               &bar[b]);
    if (le > ls)
      bulk_g2s(lbuf(b), reinterpret_cast<const unsigned char *>(lidx) + ls, (uint32_t)(le - ls),
               &bar[b]);
  };
  if (lane == 0)
    for (int k = 0; k < NST - 1 && k < my; ++k) issue(gw + k * nw, k);
  const int gl = lane & (G - 1);
  const unsigned mask = group_mask<G>();
  DotAcc<float> acc;
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
    const int64_t r0 = tile * RW, r1 = min((int64_t)n, r0 + RW);
    const uint32_t u0 = urp[r0], u1 = urp[r1], l0 = lrp[r0], l1 = lrp[r1];
    // capu / capl are the largest tile's counts, so every tile is staged;
    // a tile that is not (a corrupted structure) is skipped and reported
    const bool staged = fits(u0, u1, l0, l1);
    if (!staged && lane == 0) atomicCAS(err, 0, 4 /* DEV_ROW_OVERFLOW */);
    const size_t vs = ((size_t)u0 * 36) & ~size_t(15);
    const size_t cs = ((size_t)u0 * 4) & ~size_t(15);
    const size_t ls = ((size_t)l0 * 8) & ~size_t(15);
    if (staged) {  // the unaligned tails (< 16 bytes each)
      const size_t ve = ((size_t)u1 * 36) & ~size_t(15), ce = ((size_t)u1 * 4) & ~size_t(15);
      const size_t le = ((size_t)l1 * 8) & ~size_t(15);
      const int vt = (int)(((size_t)u1 * 36 - ve) / 4);
      const int ct = (int)(((size_t)u1 * 4 - ce) / 4);
      const int lt = (int)(((size_t)l1 * 8 - le) / 4);
      if (lane < vt) vbuf(b)[(ve - vs) / 4 + lane] = uv[ve / 4 + lane];
      if (lane >= 8 && lane < 8 + ct) cbuf(b)[(ce - cs) / 4 + lane - 8] = ucol[ce / 4 + lane - 8];
      if (lane >= 16 && lane < 16 + lt)
        reinterpret_cast<uint32_t *>(lbuf(b))[(le - ls) / 4 + lane - 16] =
            reinterpret_cast<const uint32_t *>(lidx)[le / 4 + lane - 16];
    }
    __syncwarp();
    const int64_t r = r0 + lane / G;
    if (r < n && staged)
      sym_row<DOT>(r, gl, mask, urp, lrp, vbuf(b), cbuf(b), lbuf(b), vs / 4, cs / 4, ls / 8, u0,
                   u1, uv, x, y, acc);
    __syncwarp();
  }
  if (DOT) {  // CG K1: the last CTA leaves the p.q total in ctl->pq_tot
    const double t = block_sum(acc.value(), shred);
    SolveCtl *c = const_cast<SolveCtl *>(ctl);
    finalize_partials(&t, 1, part, &c->tick1, &c->pq_tot, shred);
  }
}

template <bool DOT, int NST> int sym_config_t(Ctx *c, SymBsr *S) {
  const size_t sh = sym_smem_bytes(S->capu, S->capl, NST);
  if (sh > 200 * 1024) return SG_ERR_UNSUPPORTED;
  auto kern = k_sbsr3_wtma<DOT, NST>;
  SG_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  int per_sm = 0;
  SG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WTMA_WARPS * 32, sh));
  if (per_sm < 1) return SG_ERR_UNSUPPORTED;
  const int64_t ntiles = ((int64_t)S->n + SYM_RW - 1) / SYM_RW;
  int64_t g = (int64_t)per_sm * c->num_sms;
  const int64_t need = (ntiles + WTMA_WARPS - 1) / WTMA_WARPS;
  if (g > need) g = need;
  if (g < 1) g = 1;
  S->grid[DOT] = (int)g;
  S->smem[DOT] = sh;
  return SG_OK;
}

template <bool DOT> int sym_config(Ctx *c, SymBsr *S) {
  switch (S->nst) {
    case 2: return sym_config_t<DOT, 2>(c, S);
    case 3: return sym_config_t<DOT, 3>(c, S);
    case 4: return sym_config_t<DOT, 4>(c, S);
    default: return SG_ERR_UNSUPPORTED;
  }
}

template <bool DOT, int NST>
void sym_launch_t(SymBsr *S, cudaStream_t st, const SolveCtl *ctl, const float *x, float *y,
                  double *part) {
  k_sbsr3_wtma<DOT, NST><<<S->grid[DOT], WTMA_WARPS * 32, S->smem[DOT], st>>>(
      ctl, S->n, S->urowptr, S->ucol, S->uvals, S->lrowptr, S->lidx, x, y, part, S->capu,
      S->capl, S->c->d_err);
}

int alloc(SymBsr *S, void **p, size_t bytes) {
  SG_CHECK_CUDA(cudaMalloc(p, bytes ? bytes : 256));
  S->allocs.push_back(*p);
  return SG_OK;
}

}  // namespace

int sym_create(Ctx *c, int32_t n, const uint32_t *rowptr, const uint32_t *colidx, int64_t nnzb,
               int stages, SymBsr *S) {
  S->c = c;
  S->nst = stages == 0 ? SYM_NST_DEFAULT : stages;
  SG_REQUIRE(S->nst >= 2 && S->nst <= 4, "symmetric storage: stages %d (2..4)", stages);
  S->n = n;
  S->nnzb = nnzb;
  S->rowptr = rowptr;
  S->colidx = colidx;
  SG_REQUIRE(n > 0 && nnzb > 0 && nnzb < 0xffffffffLL / 9, "symmetric storage: n %d nnzb %lld",
             n, (long long)nnzb);
  SG_TRY(alloc(S, (void **)&S->dslot, (size_t)n * 4));
  SG_TRY(alloc(S, (void **)&S->urowptr, (size_t)(n + 1) * 4));
  SG_TRY(alloc(S, (void **)&S->lrowptr, (size_t)(n + 1) * 4));
  {
    Scratch s(c);
    SG_TRY(s.reserve((size_t)n * 8 + 2 * scan_scratch_bytes(n) + 1024));
    uint32_t *ucnt = s.alloc<uint32_t>(n), *lcnt = s.alloc<uint32_t>(n);
    const int g = grid_for(c, n, 256, 8);
    k_sym_count<<<g, 256, 0, c->stream>>>(n, rowptr, colidx, S->dslot, ucnt, lcnt, c->d_err);
    SG_CHECK_LAUNCH();
    SG_TRY(exclusive_scan_u32(c, s, ucnt, S->urowptr, n));
    SG_TRY(exclusive_scan_u32(c, s, lcnt, S->lrowptr, n));
    SG_TRY(check_device_error(c, "symmetric storage (diagonal blocks)"));
  }
  uint32_t tot[2];
  SG_CHECK_CUDA(cudaMemcpyAsync(&tot[0], S->urowptr + n, 4, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaMemcpyAsync(&tot[1], S->lrowptr + n, 4, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  S->nu = tot[0];
  S->nl = tot[1];
  SG_REQUIRE(S->nu + S->nl == nnzb, "symmetric storage: %lld + %lld blocks != nnzb %lld",
             (long long)S->nu, (long long)S->nl, (long long)nnzb);
  // a symmetric pattern has as many blocks below the diagonal as above it
  // (with every lower block's mirror found below, the two halves then match)
  if (S->nu - n != S->nl)
    return set_error(SG_ERR_ARG, "symmetric storage: %lld blocks above the diagonal, %lld below",
                     (long long)(S->nu - n), (long long)S->nl);
  SG_TRY(alloc(S, (void **)&S->ucol, (size_t)S->nu * 4));
  SG_TRY(alloc(S, (void **)&S->lidx, (size_t)S->nl * 8));
  SG_TRY(alloc(S, (void **)&S->uvals, (size_t)S->nu * 36));
  const int g = grid_for(c, n, 256, 8);
  k_sym_pattern<<<g, 256, 0, c->stream>>>(n, rowptr, colidx, S->dslot, S->urowptr, S->lrowptr,
                                           S->ucol, S->lidx, c->d_err);
  SG_CHECK_LAUNCH();
  SG_TRY(check_device_error(c, "symmetric storage (pattern not symmetric)"));
  unsigned *dmax = nullptr;
  SG_TRY(alloc(S, (void **)&dmax, 8));
  SG_CHECK_CUDA(cudaMemsetAsync(dmax, 0, 8, c->stream));
  k_tile_max<<<g, 256, 0, c->stream>>>(n, S->urowptr, SYM_RW, dmax);
  k_tile_max<<<g, 256, 0, c->stream>>>(n, S->lrowptr, SYM_RW, dmax + 1);
  SG_CHECK_LAUNCH();
  unsigned caps[2];
  SG_CHECK_CUDA(cudaMemcpyAsync(caps, dmax, 8, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  S->capu = (int)caps[0];
  S->capl = (int)caps[1] > 0 ? (int)caps[1] : 1;
  if (sym_config<true>(c, S) != SG_OK || sym_config<false>(c, S) != SG_OK)
    return set_error(SG_ERR_UNSUPPORTED,
                     "symmetric storage: warp tiles of %d upper / %d lower blocks exceed shared "
                     "memory", S->capu, S->capl);
  return SG_OK;
}

int sym_fill(SymBsr *S, cudaStream_t st, const float *vals) {
  k_sym_copy<<<grid_for(S->c, (int64_t)S->n * 32, 256, 8), 256, 0, st>>>(
      S->n, S->rowptr, S->dslot, S->urowptr, vals, S->uvals);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

int sym_launch(SymBsr *S, cudaStream_t st, const SolveCtl *ctl, bool dot, const float *x,
               float *y, double *part) {
  switch (S->nst * 2 + (dot ? 1 : 0)) {
    case 4: sym_launch_t<false, 2>(S, st, nullptr, x, y, part); break;
    case 5: sym_launch_t<true, 2>(S, st, ctl, x, y, part); break;
    case 6: sym_launch_t<false, 3>(S, st, nullptr, x, y, part); break;
    case 7: sym_launch_t<true, 3>(S, st, ctl, x, y, part); break;
    case 8: sym_launch_t<false, 4>(S, st, nullptr, x, y, part); break;
    default: sym_launch_t<true, 4>(S, st, ctl, x, y, part); break;
  }
  SG_CHECK_LAUNCH();
  return SG_OK;
}

void sym_free(SymBsr *S) {
  if (!S) return;
  for (void *p : S->allocs) cudaFree(p);
  S->allocs.clear();
}

}  // namespace sg

using namespace sg;

extern "C" {

int sg_symbsr_create(sg_ctx *h, int32_t n, const uint32_t *rowptr, const uint32_t *colidx,
                     int64_t nnzb, int32_t stages, sg_symbsr **out) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && out && rowptr && colidx, "sg_symbsr_create: null argument");
  auto *S = new SymBsr();
  const int rc = sym_create(c, n, rowptr, colidx, nnzb, stages, S);
  if (rc != SG_OK) {
    sym_free(S);
    delete S;
    return rc;
  }
  ctx_retain(c);
  *out = reinterpret_cast<sg_symbsr *>(S);
  return SG_OK;
}

int sg_symbsr_fill(sg_symbsr *h, const float *vals) {
  SymBsr *S = reinterpret_cast<SymBsr *>(h);
  DeviceGuard dg_(S ? S->c : nullptr);
  SG_REQUIRE(S && vals, "sg_symbsr_fill: null argument");
  return sym_fill(S, S->c->stream, vals);
}

int sg_symbsr_spmv(sg_symbsr *h, const float *x, float *y) {
  SymBsr *S = reinterpret_cast<SymBsr *>(h);
  DeviceGuard dg_(S ? S->c : nullptr);
  SG_REQUIRE(S && x && y, "sg_symbsr_spmv: null argument");
  return sym_launch(S, S->c->stream, nullptr, false, x, y, nullptr);
}

int sg_symbsr_destroy(sg_symbsr *h) {
  SymBsr *S = reinterpret_cast<SymBsr *>(h);
  DeviceGuard dg_(S ? S->c : nullptr);
  if (!S) return SG_OK;
  Ctx *c = S->c;
  cudaStreamSynchronize(c->stream);
  sym_free(S);
  delete S;
  ctx_release(c);
  return SG_OK;
}

}  // extern "C"
