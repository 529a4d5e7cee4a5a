// sg_bspmv: blocked SpMV entry point (y = A x) and its lanes-per-row choice.
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "sg_internal.cuh"
#include "sg_spmv.cuh"
#include "sg_spmv_tma.cuh"
#include "sg_spmv_api.h"

namespace sg {

// TMA SpMV variants: (lanes per block row, rows per CTA tile, pipeline
// stages); ROWS <= 0 selects the per-warp pipeline with warp tiles of
// max(1, -ROWS) passes of 32/G rows (passes > 1 only for scalar CSR; for
// 3x3 blocks those variants run one pass).
struct TmaVariant {
  int G, ROWS, NST;
};
static const TmaVariant kTmaVariants[] = {
    {8, 32, 2}, {8, 32, 3}, {8, 16, 4}, {4, 32, 3}, {16, 16, 4}, {8, 16, 2},
    {8, 0, 2},  {8, 0, 3},  {8, 0, 4},  {4, 0, 2},  {4, 0, 3},  {2, 0, 2},
    {4, -4, 2}, {4, -8, 2}, {8, -8, 2},
};
constexpr int kNumTmaVariants = sizeof(kTmaVariants) / sizeof(kTmaVariants[0]);
// The variant g = 0 (and the solver) use: the fastest on the 128^3 lattice.
constexpr int kDefaultTmaVariant = 9;   // 3x3: per-warp, 4 lanes per row, 2 stages
constexpr int kDefaultTmaVariant1 = 12; // scalar: per-warp, 4 lanes, 4 passes (32 rows)
int default_tma_variant(int bs) { return bs == 1 ? kDefaultTmaVariant1 : kDefaultTmaVariant; }

// Blocks in the largest tile of `rows` consecutive rows (the buffer size).
static int tile_cap(int rows, const PatternStats &ps) {
  const int bound = rows * (ps.maxrow > 0 ? ps.maxrow : 1);
  const int t = rows == 16 ? ps.tile16
              : rows == 32 ? ps.tile32
              : rows == 4  ? ps.tile4
              : rows == 8  ? ps.tile8 : 0;
  return (t > 0 && t < bound) ? t : bound;
}

template <int G, int ROWS, int NST, typename MT, typename VT, bool DOT>
static int tma_config_t(Ctx *c, int32_t n, const PatternStats &ps, int *grid, size_t *smem) {
  const int capb = tile_cap(ROWS, ps);
  const size_t sh = tma_smem_bytes<MT>(capb, NST);
  if (sh > 200 * 1024) return SG_ERR_UNSUPPORTED;
  auto kern = k_bsr3_tma<G, ROWS, NST, MT, VT, DOT>;
  SG_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  int per_sm = 0;
  SG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, ROWS * G, sh));
  if (per_sm < 1) return SG_ERR_UNSUPPORTED;
  const int ntiles = (n + ROWS - 1) / ROWS;
  int gsz = per_sm * c->num_sms;
  if (gsz > ntiles) gsz = ntiles;
  if (gsz < 1) gsz = 1;
  *grid = gsz;
  *smem = sh;
  return SG_OK;
}

template <int G, int ROWS, int NST, typename MT, typename VT, bool DOT>
static int tma_launch_t(Ctx *c, cudaStream_t st, const SolveCtl *ctl, int32_t n,
                        const uint32_t *rp, const uint32_t *ci, const MT *v, const VT *x, VT *y,
                        double *part, const PatternStats &ps, int grid, size_t smem) {
  const int capb = tile_cap(ROWS, ps);
  k_bsr3_tma<G, ROWS, NST, MT, VT, DOT><<<grid, ROWS * G, smem, st>>>(ctl, n, rp, ci, v, x, y,
                                                                      part, capb, c->d_err);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <int BS, int G, int NST, int P, typename MT, typename VT, bool DOT>
static int wtma_config_t(Ctx *c, int32_t n, const PatternStats &ps, int *grid, size_t *smem) {
  const int rows = 32 / G * P;
  const int capb = tile_cap(rows, ps);
  const size_t sh = wtma_smem_bytes<MT, BS * BS>(capb, NST);
  if (sh > 200 * 1024) return SG_ERR_UNSUPPORTED;
  auto kern = BS == 3 ? k_bsr3_wtma<G, NST, MT, VT, DOT> : k_csr_wtma<G, NST, P, MT, VT, DOT>;
  SG_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  int per_sm = 0;
  SG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WTMA_WARPS * 32, sh));
  if (per_sm < 1) return SG_ERR_UNSUPPORTED;
  const int64_t ntiles = ((int64_t)n + rows - 1) / rows;
  int64_t gsz = (int64_t)per_sm * c->num_sms;
  const int64_t need = (ntiles + WTMA_WARPS - 1) / WTMA_WARPS;
  if (gsz > need) gsz = need;
  if (gsz < 1) gsz = 1;
  *grid = (int)gsz;
  *smem = sh;
  return SG_OK;
}

template <int BS, int G, int NST, int P, typename MT, typename VT, bool DOT>
static int wtma_launch_t(Ctx *c, cudaStream_t st, const SolveCtl *ctl, int32_t n,
                         const uint32_t *rp, const uint32_t *ci, const MT *v, const VT *x, VT *y,
                         double *part, const PatternStats &ps, int grid, size_t smem) {
  const int capb = tile_cap(32 / G * P, ps);
  // launch_k: inside a solver's graph capture the launch may overlap the
  // previous kernel's tail (the kernel waits for it before any access)
  if (BS == 3)
    SG_CHECK_CUDA(launch_k(c, k_bsr3_wtma<G, NST, MT, VT, DOT>, grid, WTMA_WARPS * 32, smem, st,
                           ctl, n, rp, ci, v, x, y, part, capb, c->d_err));
  else
    SG_CHECK_CUDA(launch_k(c, k_csr_wtma<G, NST, P, MT, VT, DOT>, grid, WTMA_WARPS * 32, smem,
                           st, ctl, n, rp, ci, v, x, y, part, capb, c->d_err));
  return SG_OK;
}

// Dispatch over (variant, dot) for one (MT, VT).
template <typename MT, typename VT>
static int tma_dispatch(Ctx *c, cudaStream_t st, bool launch, int bs, int var, int dot,
                        const SolveCtl *ctl, int32_t n, const uint32_t *rp, const uint32_t *ci,
                        const void *v, const void *x, void *y, double *part,
                        const PatternStats &ps, int *grid, size_t *smem) {
#define SG_V(ID, G, R, N)                                                                      \
  case ID:                                                                                     \
    if (bs != 3) return SG_ERR_UNSUPPORTED;                                                    \
    if (launch)                                                                                \
      return dot ? tma_launch_t<G, R, N, MT, VT, true>(c, st, ctl, n, rp, ci, (const MT *)v,   \
                                                       (const VT *)x, (VT *)y, part, ps,       \
                                                       *grid, *smem)                           \
                 : tma_launch_t<G, R, N, MT, VT, false>(c, st, ctl, n, rp, ci, (const MT *)v,  \
                                                        (const VT *)x, (VT *)y, part, ps,      \
                                                        *grid, *smem);                         \
    return dot ? tma_config_t<G, R, N, MT, VT, true>(c, n, ps, grid, smem)                     \
               : tma_config_t<G, R, N, MT, VT, false>(c, n, ps, grid, smem);
  switch (var) {
    SG_V(0, 8, 32, 2)
    SG_V(1, 8, 32, 3)
    SG_V(2, 8, 16, 4)
    SG_V(3, 4, 32, 3)
    SG_V(4, 16, 16, 4)
    SG_V(5, 8, 16, 2)
#define SG_W1(ID, BS, G, N, P)                                                                    \
    if (launch)                                                                                \
      return dot ? wtma_launch_t<BS, G, N, P, MT, VT, true>(c, st, ctl, n, rp, ci, (const MT *)v, \
                                                         (const VT *)x, (VT *)y, part, ps,     \
                                                         *grid, *smem)                         \
                 : wtma_launch_t<BS, G, N, P, MT, VT, false>(c, st, ctl, n, rp, ci,               \
                                                          (const MT *)v, (const VT *)x,        \
                                                          (VT *)y, part, ps, *grid, *smem);    \
    return dot ? wtma_config_t<BS, G, N, P, MT, VT, true>(c, n, ps, grid, smem)                   \
               : wtma_config_t<BS, G, N, P, MT, VT, false>(c, n, ps, grid, smem);
#define SG_W(ID, G, N, P)                                                                      \
  case ID:                                                                                     \
    if (bs == 3) {                                                                             \
      SG_W1(ID, 3, G, N, 1)                                                                    \
    } else {                                                                                   \
      SG_W1(ID, 1, G, N, P)                                                                    \
    }
    SG_W(6, 8, 2, 1)
    SG_W(7, 8, 3, 1)
    SG_W(8, 8, 4, 1)
    SG_W(9, 4, 2, 1)
    SG_W(10, 4, 3, 1)
    SG_W(11, 2, 2, 1)
    SG_W(12, 4, 2, 4)
    SG_W(13, 4, 2, 8)
    SG_W(14, 8, 2, 8)
    default: return SG_ERR_ARG;
  }
#undef SG_V
#undef SG_W
#undef SG_W1
}

static int tma_any(Ctx *c, cudaStream_t st, bool launch, int bs, int vdt, int xdt, int var, int dot,
                   const void *ctl, int32_t n, const uint32_t *rp, const uint32_t *ci,
                   const void *v, const void *x, void *y, double *part, const PatternStats &ps,
                   int *grid, size_t *smem) {
  const SolveCtl *k = (const SolveCtl *)ctl;
  if (vdt == SG_F32 && xdt == SG_F32)
    return tma_dispatch<float, float>(c, st, launch, bs, var, dot, k, n, rp, ci, v, x, y, part, ps,
                                      grid, smem);
  if (vdt == SG_F64 && xdt == SG_F64)
    return tma_dispatch<double, double>(c, st, launch, bs, var, dot, k, n, rp, ci, v, x, y, part, ps,
                                        grid, smem);
  if (vdt == SG_F32 && xdt == SG_F64)
    return tma_dispatch<float, double>(c, st, launch, bs, var, dot, k, n, rp, ci, v, x, y, part, ps,
                                       grid, smem);
  return SG_ERR_UNSUPPORTED;
}

int bsr3_tma_config(Ctx *c, int bs, int vdt, int xdt, int var, int dot, int32_t n,
                    const PatternStats &ps, int *grid, size_t *smem) {
  return tma_any(c, nullptr, false, bs, vdt, xdt, var, dot, nullptr, n, nullptr, nullptr, nullptr,
                 nullptr, nullptr, nullptr, ps, grid, smem);
}

int bsr3_tma_launch(Ctx *c, cudaStream_t st, const void *ctl, int bs, int vdt, int xdt, int var,
                    int dot, int32_t n, const uint32_t *rp, const uint32_t *ci, const void *v,
                    const void *x, void *y, double *part, const PatternStats &ps, int grid,
                    size_t smem) {
  return tma_any(c, st, true, bs, vdt, xdt, var, dot, ctl, n, rp, ci, v, x, y, part, ps, &grid,
                 &smem);
}

// Longest row and largest 16- / 32-row tiles (blocks) of a pattern.
__global__ void k_pattern_stats(const uint32_t *rowptr, int32_t n, uint32_t *out) {
  uint32_t mr = 0, t16 = 0, t32 = 0, t4 = 0, t8 = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    mr = max(mr, rowptr[i + 1] - rowptr[i]);
    if (i % 16 == 0) t16 = max(t16, rowptr[min((int64_t)n, i + 16)] - rowptr[i]);
    if (i % 32 == 0) t32 = max(t32, rowptr[min((int64_t)n, i + 32)] - rowptr[i]);
    if (i % 4 == 0) t4 = max(t4, rowptr[min((int64_t)n, i + 4)] - rowptr[i]);
    if (i % 8 == 0) t8 = max(t8, rowptr[min((int64_t)n, i + 8)] - rowptr[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mr = max(mr, __shfl_down_sync(0xffffffffu, mr, o));
    t16 = max(t16, __shfl_down_sync(0xffffffffu, t16, o));
    t32 = max(t32, __shfl_down_sync(0xffffffffu, t32, o));
    t4 = max(t4, __shfl_down_sync(0xffffffffu, t4, o));
    t8 = max(t8, __shfl_down_sync(0xffffffffu, t8, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], mr);
    atomicMax(&out[1], t16);
    atomicMax(&out[2], t32);
    atomicMax(&out[3], t4);
    atomicMax(&out[4], t8);
  }
}

// Pattern statistics, cached per (rowptr, n).  The cache cannot see a new
// pattern written at the same address, so callers that own a pattern for a
// long time (the solver) pass refresh = true; the SpMV kernels never rely on
// the statistics for memory safety (a tile larger than the buffers is read
// straight from global memory).
int cached_stats(Ctx *c, int32_t n, const uint32_t *rowptr, PatternStats *ps, bool refresh) {
  int slot = -1;
  for (int i = 0; i < Ctx::MAXROW_CACHE; ++i)
    if (c->mr_ptr[i] == rowptr && c->mr_n[i] == n) slot = i;
  if (slot >= 0 && !refresh) {
    ps->maxrow = c->mr_val[slot];
    ps->tile16 = c->mr_t16[slot];
    ps->tile32 = c->mr_t32[slot];
    ps->tile4 = c->mr_t4[slot];
    ps->tile8 = c->mr_t8[slot];
    return SG_OK;
  }
  Scratch s(c);
  SG_TRY(s.reserve(256));
  uint32_t *d = s.alloc<uint32_t>(8);
  SG_CHECK_CUDA(cudaMemsetAsync(d, 0, 32, c->stream));
  if (n > 0) {
    k_pattern_stats<<<grid_for(c, n, 256, 4), 256, 0, c->stream>>>(rowptr, n, d);
    SG_CHECK_LAUNCH();
  }
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, d, 32, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  const uint32_t *h = (const uint32_t *)c->h_stage;
  if (slot < 0) slot = c->mr_next++ % Ctx::MAXROW_CACHE;
  c->mr_ptr[slot] = rowptr;
  c->mr_n[slot] = n;
  c->mr_val[slot] = ps->maxrow = (int32_t)h[0];
  c->mr_t16[slot] = ps->tile16 = (int32_t)h[1];
  c->mr_t32[slot] = ps->tile32 = (int32_t)h[2];
  c->mr_t4[slot] = ps->tile4 = (int32_t)h[3];
  c->mr_t8[slot] = ps->tile8 = (int32_t)h[4];
  return SG_OK;
}

int cached_maxrow(Ctx *c, int32_t n, const uint32_t *rowptr, int *out) {
  PatternStats ps;
  SG_TRY(cached_stats(c, n, rowptr, &ps));
  *out = ps.maxrow;
  return SG_OK;
}

template <int G, typename VT, typename XT, typename AT>
__global__ void __launch_bounds__(256) k_bsr3(int32_t n, const uint32_t *__restrict__ rowptr,
                                              const uint32_t *__restrict__ colidx,
                                              const VT *__restrict__ vals,
                                              const XT *__restrict__ x, XT *__restrict__ y) {
  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = group_mask<G>();
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x / G);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; r < n; r += stride) {
    AT y0, y1, y2;
    bsr3_row<G, VT, XT, AT>(rowptr, colidx, vals, x, r, gl, mask, y0, y1, y2);
    if (G >= 3) {
      if (gl < 3) y[r * 3 + gl] = (XT)(gl == 0 ? y0 : (gl == 1 ? y1 : y2));
    } else if (gl == 0) {
      y[r * 3 + 0] = (XT)y0;
      y[r * 3 + 1] = (XT)y1;
      y[r * 3 + 2] = (XT)y2;
    }
  }
}

template <int G, typename VT, typename XT, typename AT>
__global__ void __launch_bounds__(256) k_csr(int32_t n, const uint32_t *__restrict__ rowptr,
                                             const uint32_t *__restrict__ colidx,
                                             const VT *__restrict__ vals,
                                             const XT *__restrict__ x, XT *__restrict__ y) {
  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = group_mask<G>();
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x / G);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; r < n; r += stride) {
    AT s = csr_row<G, VT, XT, AT>(rowptr, colidx, vals, x, r, gl, mask);
    if (gl == 0) y[r] = (XT)s;
  }
}

template <int G, int BS, typename VT, typename XT, typename AT>
__global__ void __launch_bounds__(256) k_bsr(int32_t n, const uint32_t *__restrict__ rowptr,
                                             const uint32_t *__restrict__ colidx,
                                             const VT *__restrict__ vals,
                                             const XT *__restrict__ x, XT *__restrict__ y) {
  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = group_mask<G>();
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x / G);
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; r < n; r += stride) {
    AT o[BS];
    bsr_row<G, BS, VT, XT, AT>(rowptr, colidx, vals, x, r, gl, mask, o);
    if (gl == 0)
      for (int i = 0; i < BS; ++i) y[r * BS + i] = (XT)o[i];
  }
}

// Any block size: one thread per block row, the lowered loop order.
template <typename VT, typename XT, typename AT>
__global__ void k_bsr_any(int32_t n, int32_t bs, const uint32_t *__restrict__ rowptr,
                          const uint32_t *__restrict__ colidx, const VT *__restrict__ vals,
                          const XT *__restrict__ x, XT *__restrict__ y) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    for (int q1 = 0; q1 < bs; ++q1) {
      AT acc = 0;
      for (uint32_t qp = rowptr[q]; qp < rowptr[q + 1]; ++qp) {
        const int64_t p = colidx[qp];
        AT t = 0;
        for (int p1 = 0; p1 < bs; ++p1)
          t += (AT)vals[(size_t)qp * bs * bs + q1 * bs + p1] * (AT)x[p * bs + p1];
        acc += t;
      }
      y[q * bs + q1] = (XT)acc;
    }
  }
}

template <typename VT, typename XT, typename AT>
static int launch_typed(Ctx *c, int32_t n, int32_t bs, const uint32_t *rp, const uint32_t *ci,
                        const VT *v, const XT *x, XT *y, int g) {
  const int T = 256;
  cudaStream_t st = c->stream;
  auto grid = [&](int G) { return grid_for(c, (int64_t)n * G, T, 8); };
#define SG_G_CASE(KERNEL, GV, ...)                                              \
  case GV:                                                                      \
    KERNEL<GV, __VA_ARGS__><<<grid(GV), T, 0, st>>>(n, rp, ci, v, x, y);        \
    break;
  if (bs == 3) {
    switch (g) {
      SG_G_CASE(k_bsr3, 1, VT, XT, AT)
      SG_G_CASE(k_bsr3, 2, VT, XT, AT)
      SG_G_CASE(k_bsr3, 4, VT, XT, AT)
      SG_G_CASE(k_bsr3, 8, VT, XT, AT)
      SG_G_CASE(k_bsr3, 16, VT, XT, AT)
      SG_G_CASE(k_bsr3, 32, VT, XT, AT)
      default: return set_error(SG_ERR_ARG, "sg_bspmv: g=%d not in {1,2,4,8,16,32}", g);
    }
  } else if (bs == 1) {
    switch (g) {
      SG_G_CASE(k_csr, 1, VT, XT, AT)
      SG_G_CASE(k_csr, 2, VT, XT, AT)
      SG_G_CASE(k_csr, 4, VT, XT, AT)
      SG_G_CASE(k_csr, 8, VT, XT, AT)
      SG_G_CASE(k_csr, 16, VT, XT, AT)
      SG_G_CASE(k_csr, 32, VT, XT, AT)
      default: return set_error(SG_ERR_ARG, "sg_bspmv: g=%d not in {1,2,4,8,16,32}", g);
    }
  } else if (bs == 2) {
    switch (g) {
      SG_G_CASE(k_bsr, 1, 2, VT, XT, AT)
      SG_G_CASE(k_bsr, 2, 2, VT, XT, AT)
      SG_G_CASE(k_bsr, 4, 2, VT, XT, AT)
      SG_G_CASE(k_bsr, 8, 2, VT, XT, AT)
      SG_G_CASE(k_bsr, 16, 2, VT, XT, AT)
      SG_G_CASE(k_bsr, 32, 2, VT, XT, AT)
      default: return set_error(SG_ERR_ARG, "sg_bspmv: g=%d not in {1,2,4,8,16,32}", g);
    }
  } else {
    k_bsr_any<VT, XT, AT><<<grid_for(c, n, T, 8), T, 0, st>>>(n, bs, rp, ci, v, x, y);
  }
#undef SG_G_CASE
  SG_CHECK_LAUNCH();
  return SG_OK;
}

int default_lanes(int32_t n, int64_t nnzb, int32_t bs) {
  const double avg = n > 0 ? (double)nnzb / n : 0.0;
  // scalar rows: few lanes per row keep more rows in flight (P1 heat 128^3,
  // 12.9 entries per row, FP64: 2 lanes 0.110 ms against 8 lanes 0.248 ms)
  if (bs == 1) return avg > 32 ? 8 : (avg > 16 ? 4 : 2);
  if (bs == 3) return avg > 24 ? 8 : 4;
  return 4;
}

int bspmv_launch(Ctx *c, int32_t n, int32_t bs, const uint32_t *rp, const uint32_t *ci,
                 int vdt, const void *v, int xdt, const void *x, void *y, int g,
                 int64_t nnzb_hint) {
  if (g == 0) g = default_lanes(n, nnzb_hint, bs);
  if (vdt == SG_F64 && xdt == SG_F64)
    return launch_typed<double, double, double>(c, n, bs, rp, ci, (const double *)v,
                                                (const double *)x, (double *)y, g);
  if (vdt == SG_F32 && xdt == SG_F32)
    return launch_typed<float, float, float>(c, n, bs, rp, ci, (const float *)v,
                                             (const float *)x, (float *)y, g);
  if (vdt == SG_F32 && xdt == SG_F64)
    return launch_typed<float, double, double>(c, n, bs, rp, ci, (const float *)v,
                                               (const double *)x, (double *)y, g);
  return set_error(SG_ERR_UNSUPPORTED, "sg_bspmv: val_dtype=%d vec_dtype=%d", vdt, xdt);
}

}  // namespace sg

using namespace sg;

extern "C" int sg_bspmv(sg_ctx *h, int32_t n, int32_t bs, const uint32_t *rowptr,
                        const uint32_t *colidx, int vdt, const void *vals, int xdt,
                        const void *x, void *y, int32_t g) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && rowptr && colidx && vals && x && y, "sg_bspmv: null argument");
  SG_REQUIRE(n >= 0 && bs >= 1 && bs <= 16, "sg_bspmv: bad n=%d bs=%d", n, bs);
  if (n == 0) return SG_OK;
  const bool aligned = ((uintptr_t)vals % 16 == 0) && ((uintptr_t)colidx % 16 == 0);
  if (g < 0) SG_REQUIRE((bs == 3 || bs == 1) && aligned && -g - 1 < kNumTmaVariants,
                        "sg_bspmv: g=%d selects TMA variant %d: bs=3 or 1, 16-byte aligned "
                        "arrays, -%d <= g <= -1", g, -g - 1, kNumTmaVariants);
  if ((g == 0 && (bs == 3 || bs == 1) && aligned && !(vdt == SG_F64 && xdt == SG_F64)) ||
      g < 0) {
    // TMA-staged kernel (lanes per row from the row length unless given).
    // FP64 matrices default to the plain kernel, which keeps more warps in
    // flight for the FP64 pipe.
    int grid = 0;
    size_t sh = 0;
    PatternStats ps;
    SG_TRY(cached_stats(c, n, rowptr, &ps));
    const int var = g < 0 ? -g - 1 : default_tma_variant(bs);
    if (bsr3_tma_config(c, bs, vdt, xdt, var, 0, n, ps, &grid, &sh) == SG_OK)
      return bsr3_tma_launch(c, c->stream, nullptr, bs, vdt, xdt, var, 0, n, rowptr, colidx, vals,
                             x, y, nullptr, ps, grid, sh);
    // the variant's buffers do not fit the largest tile (very long rows):
    // the streaming G-lane kernel needs no staging
    g = 0;
  }
  // nnzb is only needed for the default lane choice; read rowptr[n] then.
  int64_t nnzb = 0;
  if (g == 0) {
    SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, rowptr + n, 4, cudaMemcpyDeviceToHost, c->stream));
    SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
    nnzb = *(uint32_t *)c->h_stage;
  }
  return bspmv_launch(c, n, bs, rowptr, colidx, vdt, vals, xdt, x, y, g, nnzb);
}

// ---------------------------------------------------------------------------
// Autotuner: every lane count / TMA variant timed on the matrix itself
// ---------------------------------------------------------------------------
namespace sg {
namespace {
using TuneKey = std::tuple<int, int32_t, int64_t, int32_t, int, int, const void *, const void *>;
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int32_t, float>> g_tune_cache;
}  // namespace
}  // namespace sg

extern "C" int sg_tune_spmv(sg_ctx *h, const sg_matrix *A, int xdt, int reps, int force,
                            int32_t *best_g, float *best_ms, float *default_ms, int32_t *ncand,
                            int32_t *cand_g, float *cand_ms, int32_t cand_cap) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && A && A->rowptr && A->colidx && A->vals && best_g && best_ms,
             "sg_tune_spmv: null argument");
  SG_REQUIRE(A->n > 0 && A->bs >= 1 && A->bs <= 16, "sg_tune_spmv: bad matrix");
  SG_REQUIRE(xdt == SG_F32 || xdt == SG_F64, "sg_tune_spmv: xdt %d", xdt);
  if (reps < 1) reps = 10;
  const TuneKey key{c->device, A->n, A->nnzb, A->bs, A->dtype, xdt, A->rowptr, A->colidx};
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      *best_g = it->second.first;
      *best_ms = it->second.second;
      if (default_ms) *default_ms = -1.f;
      if (ncand) *ncand = 0;
      return SG_OK;
    }
  }
  // candidates: the default (g = 0) first, then every TMA variant the matrix
  // admits, then every streaming lane count
  std::vector<int32_t> cands{0};
  const bool aligned = ((uintptr_t)A->vals % 16 == 0) && ((uintptr_t)A->colidx % 16 == 0);
  if ((A->bs == 3 || A->bs == 1) && aligned)
    for (int v = 0; v < kNumTmaVariants; ++v) cands.push_back(-(v + 1));
  for (int g : {1, 2, 4, 8, 16, 32}) cands.push_back(g);
  const size_t xb = (size_t)A->n * A->bs * dtype_size(xdt);
  // x and y from the context arena (contents irrelevant: zeroed)
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(xb, 1) * 2 + 512));
  unsigned char *x = s.alloc<unsigned char>(xb), *y = s.alloc<unsigned char>(xb);
  SG_CHECK_CUDA(cudaMemsetAsync(x, 0, xb, c->stream));
  cudaEvent_t e0, e1;
  SG_CHECK_CUDA(cudaEventCreate(&e0));
  SG_CHECK_CUDA(cudaEventCreate(&e1));
  int32_t bg = 0;
  float bms = 0.f, dms = 0.f;
  int nc = 0;
  int rc = SG_OK;
  for (int32_t g : cands) {
    rc = sg_bspmv(h, A->n, A->bs, A->rowptr, A->colidx, A->dtype, A->vals, xdt, x, y, g);
    if (rc != SG_OK) break;
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && rc == SG_OK; ++r)
      rc = sg_bspmv(h, A->n, A->bs, A->rowptr, A->colidx, A->dtype, A->vals, xdt, x, y, g);
    cudaEventRecord(e1, c->stream);
    if (rc != SG_OK) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = set_error(SG_ERR_CUDA, "sg_tune_spmv: event wait failed");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= reps;
    if (g == 0) dms = ms;
    if (nc == 0 || ms < bms) {
      bms = ms;
      bg = g;
    }
    if (cand_g && cand_ms && nc < cand_cap) {
      cand_g[nc] = g;
      cand_ms[nc] = ms;
    }
    ++nc;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  SG_TRY(rc);
  SG_TRY(check_device_error(c, "sg_tune_spmv"));
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = {bg, bms};
  }
  *best_g = bg;
  *best_ms = bms;
  if (default_ms) *default_ms = dms;
  if (ncand) *ncand = nc;
  return SG_OK;
}
