// Learned (message-passing) preconditioner: graph data, forward, backward,
// loss, optimiser and the flexible-PCG hook.  Definitions in sg_mpnn.cuh.
#include <math.h>

#include "sg_internal.cuh"
#include "sg_mpnn_fold.cuh"
#include "sg_mpnn_fwd.cuh"
#include "sg_solver.h"
#include "sg_spmv_api.h"

namespace sg {
namespace mpnn {

struct GraphH {
  Ctx *c = nullptr;
  Graph g;
  std::vector<void *> allocs;
  bool train_ready = false;
  // symmetric form: a second set of layer buffers over the same graph data
  // (the transposed network's pass, and the second training forward)
  GraphH *twin = nullptr;
  // folded evaluation of the symmetric form (sg_mpnn_fold.cuh): its buffers
  // (allocated on first use), the sliced-ELLPACK pattern with FP16 and FP32
  // edge weights in slice order, packed L^-1
  int exec = SG_MPNN_EXEC_LAYERED;  // how sg_mpnn_forward evaluates (train = 0)
  bool fold_ready = false;
  FoldBufs fb{};
  float *fold = nullptr;
  __half *ah = nullptr;
  float *af = nullptr;
  int64_t sl_total = 0;
};

static int galloc(GraphH *G, void **p, size_t bytes) {
  SG_CHECK_CUDA(cudaMalloc(p, bytes < 256 ? 256 : bytes));
  G->allocs.push_back(*p);
  return SG_OK;
}

static void graph_free(GraphH *G) {
  if (!G) return;
  graph_free(G->twin);
  for (void *p : G->allocs) cudaFree(p);
  delete G;
}

// ---------------------------------------------------------------------------
// backward (FP32, one warp per vertex; training meshes only)
// ---------------------------------------------------------------------------
// B1: dg3 = (Wout^T dz) * [g3 > 0]; dm3 = W3m^T dg3; dh2a = bf(W3h)^T dg3.
__global__ void k_b1(int32_t n, int lin, const float *__restrict__ prm, const float *__restrict__ dz,
                     const float *__restrict__ g3, float *__restrict__ dg3,
                     float *__restrict__ dm3, float *__restrict__ dh2a) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = wid; v < n; v += nw) {
    const float d0 = dz[v * 3], d1 = dz[v * 3 + 1], d2 = dz[v * 3 + 2];
    float dg[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int h = lane * 2 + e;
      const float d = prm[O_WOUT + h] * d0 + prm[O_WOUT + H + h] * d1 + prm[O_WOUT + 2 * H + h] * d2;
      dg[e] = (lin || g3[v * H + h] > 0.f) ? d : 0.f;
      dg3[v * H + h] = dg[e];
    }
    // dm3_j = sum_h W3m[h][j] dg3[h]
#pragma unroll
    for (int j = 0; j < K; ++j) {
      float p = prm[O_W3M + (lane * 2) * K + j] * dg[0] + prm[O_W3M + (lane * 2 + 1) * K + j] * dg[1];
      for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
      if (lane == 0) dm3[v * K + j] = p;
    }
    // dh2a[c] = sum_h bf(W3h[h][c]) dg3[h]; lane owns c = 2*lane + e
    float acc0 = 0.f, acc1 = 0.f;
    for (int h = 0; h < H; ++h) {
      const float dgh = __shfl_sync(0xffffffffu, dg[h & 1], h >> 1);
      acc0 += bf16r(prm[O_W3H + h * H + lane * 2]) * dgh;
      acc1 += bf16r(prm[O_W3H + h * H + lane * 2 + 1]) * dgh;
    }
    dh2a[v * H + lane * 2] = acc0;
    dh2a[v * H + lane * 2 + 1] = acc1;
  }
}

// Generic middle step: dq = sum_u a dm_u (K); dh = dha + P^T dq; dg = dh *
// [g > 0]; optional dm_next = Wm^T dg (K), dha_next = bf(Wh)^T dg (H).
__global__ void k_bmid(int32_t n, int lin, const uint32_t *__restrict__ rowptr,
                       const uint32_t *__restrict__ colidx, const float *__restrict__ a,
                       const float *__restrict__ prm, int oP, int oWm, int oWh,
                       const float *__restrict__ dm, const float *__restrict__ dha,
                       const float *__restrict__ g, float *__restrict__ dq,
                       float *__restrict__ dgout, float *__restrict__ dm_next,
                       float *__restrict__ dha_next) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t v = wid; v < n; v += nw) {
    // dq (K values): lanes 0..7 gather one component each
    float dqj = 0.f;
    if (lane < K)
      for (uint32_t q = rowptr[v]; q < rowptr[v + 1]; ++q) dqj += a[q] * dm[(size_t)colidx[q] * K + lane];
    if (lane < K) dq[v * K + lane] = dqj;
    float dg[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int h = lane * 2 + e;
      float d = dha[v * H + h];
#pragma unroll
      for (int j = 0; j < K; ++j) d += prm[oP + j * H + h] * __shfl_sync(0xffffffffu, dqj, j);
      dg[e] = (lin || g[v * H + h] > 0.f) ? d : 0.f;
      dgout[v * H + h] = dg[e];
    }
    if (dm_next) {
#pragma unroll
      for (int j = 0; j < K; ++j) {
        float p = prm[oWm + (lane * 2) * K + j] * dg[0] + prm[oWm + (lane * 2 + 1) * K + j] * dg[1];
        for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        if (lane == 0) dm_next[v * K + j] = p;
      }
      float acc0 = 0.f, acc1 = 0.f;
      for (int h = 0; h < H; ++h) {
        const float dgh = __shfl_sync(0xffffffffu, dg[h & 1], h >> 1);
        acc0 += bf16r(prm[oWh + h * H + lane * 2]) * dgh;
        acc1 += bf16r(prm[oWh + h * H + lane * 2 + 1]) * dgh;
      }
      dha_next[v * H + lane * 2] = acc0;
      dha_next[v * H + lane * 2 + 1] = acc1;
    }
  }
}

// Outer-product reduction dW[o][i] = sum_v X_v[o] * Y_v[i] over a chunk of
// vertices per CTA; partials part[chunk][O*I], summed in order afterwards.
// Y is transformed: 0 identity, 1 relu, 2 bf16(relu), 4 bf16.
constexpr int OUTER_CHUNK = 1024;
__global__ void k_outer(int32_t n, const float *__restrict__ X, int O, const float *__restrict__ Y,
                        int I, int ytr, float *__restrict__ part) {
  const int64_t v0 = (int64_t)blockIdx.x * OUTER_CHUNK;
  const int64_t v1 = min((int64_t)n, v0 + OUTER_CHUNK);
  for (int e = threadIdx.x; e < O * I; e += blockDim.x) {
    const int o = e / I, i = e % I;
    float acc = 0.f;
    for (int64_t v = v0; v < v1; ++v) {
      float y = Y[v * I + i];
      if (ytr == 1 || ytr == 2) y = fmaxf(y, 0.f);
      if (ytr == 2 || ytr == 4) y = bf16r(y);
      acc += X[v * O + o] * y;
    }
    part[(size_t)blockIdx.x * O * I + e] = acc;
  }
}

__global__ void k_outer_sum(const float *__restrict__ part, int chunks, int len,
                            float *__restrict__ out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < len; e += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < chunks; ++c) s += part[(size_t)c * len + e];
    out[e] = s;
  }
}

__global__ void k_adam(int np, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += gridDim.x * blockDim.x) {
    const float gi = isfinite(g[i]) ? g[i] : 0.f;
    m[i] = b1 * m[i] + (1.f - b1) * gi;
    v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
    p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
  }
}

// d = z - e
__global__ void k_sub(int64_t len, const float *a, const float *b, float *d) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    d[i] = a[i] - b[i];
}
__global__ void k_scale(int64_t len, const float *a, float s, float *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = s * a[i];
}

// rz = r.z and zq = z.q partials for the CG's K3 (grid = P2 blocks).
__global__ void __launch_bounds__(RED_T) k_rz_zq(const SolveCtl *ctl, int64_t len,
                                                 const float *__restrict__ r,
                                                 const float *__restrict__ z,
                                                 const float *__restrict__ q,
                                                 double *__restrict__ part) {
  __shared__ double sh[33];
  if (ctl && ctl->status != ST_RUNNING) return;
  DotAcc<float> rz, zq;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    rz.add(r[i], z[i]);
    zq.add(z[i], q[i]);
  }
  const double t0 = block_sum(rz.value(), sh);
  const double t1 = block_sum(zq.value(), sh);
  if (threadIdx.x == 0) {
    part[gridDim.x + blockIdx.x] = t0;
    part[2 * gridDim.x + blockIdx.x] = t1;
  }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------
static int graph_refresh(GraphH *G) {
  Ctx *c = G->c;
  Graph &g = G->g;
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(g.n, 4) + 256));
  float *dn = s.alloc<float>(g.n);
  const int gr = grid_for(c, g.n, 256, 8);
  if (g.vdt == SG_F64) {
    k_diag_norm<double><<<gr, 256, 0, c->stream>>>(g.n, g.rowptr, g.colidx, (const double *)g.vals, dn);
    k_edge_weights<double><<<gr, 256, 0, c->stream>>>(g.n, g.rowptr, g.colidx, (const double *)g.vals, dn, g.a);
    k_diag_inv<double, float><<<gr, 256, 0, c->stream>>>(g.n, 3, g.rowptr, g.colidx, (const double *)g.vals, g.dinv, 1, c->d_err);
  } else {
    k_diag_norm<float><<<gr, 256, 0, c->stream>>>(g.n, g.rowptr, g.colidx, (const float *)g.vals, dn);
    k_edge_weights<float><<<gr, 256, 0, c->stream>>>(g.n, g.rowptr, g.colidx, (const float *)g.vals, dn, g.a);
    k_diag_inv<float, float><<<gr, 256, 0, c->stream>>>(g.n, 3, g.rowptr, g.colidx, (const float *)g.vals, g.dinv, 1, c->d_err);
  }
  if (g.linv) {
    if (g.vdt == SG_F64)
      k_chol_inv<double><<<gr, 256, 0, c->stream>>>(g.n, g.rowptr, g.colidx, (const double *)g.vals, g.linv);
    else
      k_chol_inv<float><<<gr, 256, 0, c->stream>>>(g.n, g.rowptr, g.colidx, (const float *)g.vals, g.linv);
  }
  SG_CHECK_LAUNCH();
  if (G->fold_ready) {
    const int ge = grid_for(c, G->sl_total, 256, 8);
    k_sell_weights<__half><<<ge, 256, 0, c->stream>>>(G->sl_total, G->fb.sl.src, g.a, G->ah);
    k_sell_weights<float><<<ge, 256, 0, c->stream>>>(G->sl_total, G->fb.sl.src, g.a, G->af);
    k_pack_linv<<<gr, 256, 0, c->stream>>>(g.n, g.linv, (float *)G->fb.l6,
                                           (uint32_t *)G->fb.l6b);
    SG_CHECK_LAUNCH();
  }
  return check_device_error(c, "mpnn graph");
}

// Layer buffers of one pass (s, m1, q2, m2, q3, m3).
static int alloc_layers(GraphH *G) {
  Graph &g = G->g;
  const size_t n = (size_t)g.n;
  SG_TRY(galloc(G, (void **)&g.s, n * 3 * 4));
  SG_TRY(galloc(G, (void **)&g.m1, n * 3 * 4));
  SG_TRY(galloc(G, (void **)&g.q2, n * K * 4));
  SG_TRY(galloc(G, (void **)&g.m2, n * K * 4));
  SG_TRY(galloc(G, (void **)&g.q3, n * K * 4));
  SG_TRY(galloc(G, (void **)&g.m3, n * K * 4));
  return SG_OK;
}

// Switch to the symmetric factorized form: L^-1, the extra vectors and the
// twin's layer buffers (allocated once).
static int set_sym(GraphH *G, int sym) {
  Graph &g = G->g;
  g.sym = sym ? 1 : 0;
  if (!sym) return SG_OK;
  g.lin = 1;
  if (G->twin) return SG_OK;
  const size_t n = (size_t)g.n;
  SG_TRY(galloc(G, (void **)&g.linv, n * 9 * 4));
  SG_TRY(galloc(G, (void **)&g.y, n * 3 * 4));
  SG_TRY(galloc(G, (void **)&g.wp, n * 3 * 4));
  SG_TRY(galloc(G, (void **)&g.t, n * 3 * 4));
  SG_TRY(galloc(G, (void **)&g.prmT, NPARAM * 4));
  SG_TRY(galloc(G, (void **)&g.gtmp, NPARAM * 4));
  GraphH *T = new GraphH();
  G->twin = T;
  T->c = G->c;
  Graph &tg = T->g;
  tg.n = g.n;
  tg.nnzb = g.nnzb;
  tg.rowptr = g.rowptr;
  tg.colidx = g.colidx;
  tg.vals = g.vals;
  tg.vdt = g.vdt;
  tg.a = g.a;
  tg.dinv = g.dinv;
  tg.linv = g.linv;
  tg.lin = 1;
  tg.sym = 1;  // split activations in its passes too (it has no twin of its own)
  SG_TRY(alloc_layers(T));
  SG_TRY(galloc(T, (void **)&tg.y, n * 3 * 4));
  SG_TRY(galloc(T, (void **)&tg.dres, 64));
  return graph_refresh(G);
}

static int graph_init(Ctx *c, const sg_matrix *A, GraphH *G) {
  SG_REQUIRE(A && A->bs == 3 && A->n > 0 && A->vals && A->rowptr && A->colidx,
             "mpnn: needs a 3x3-blocked matrix");
  G->c = c;
  Graph &g = G->g;
  g.n = A->n;
  g.nnzb = A->nnzb;
  g.rowptr = A->rowptr;
  g.colidx = A->colidx;
  g.vals = A->vals;
  g.vdt = A->dtype;
  const size_t n = (size_t)A->n;
  SG_TRY(galloc(G, (void **)&g.a, A->nnzb * 4));
  SG_TRY(galloc(G, (void **)&g.dinv, n * 9 * 4));
  SG_TRY(alloc_layers(G));
  SG_TRY(galloc(G, (void **)&g.dres, 64));
  static PerDeviceOnce attr;
  SG_TRY(once_per_device(attr, c->device, []() -> int {
    SG_CHECK_CUDA(cudaFuncSetAttribute(k_f3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
    SG_CHECK_CUDA(cudaFuncSetAttribute(k_f4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_smem_bytes()));
    return SG_OK;
  }));
  return graph_refresh(G);
}

// Buffers and graph data of the folded evaluation (symmetric form only).
static int ensure_folded(GraphH *G) {
  if (G->fold_ready) return SG_OK;
  Graph &g = G->g;
  SG_REQUIRE(g.sym && g.linv, "mpnn: the folded evaluation needs the symmetric form");
  const size_t n = (size_t)g.n;
  Ctx *c = G->c;
  FoldBufs &B = G->fb;
  float *l6 = nullptr;
  uint32_t *l6b = nullptr;
  SG_TRY(galloc(G, (void **)&G->fold, NPOLY * 9 * 4));
  SG_TRY(galloc(G, (void **)&l6, n * 6 * 4));
  SG_TRY(galloc(G, (void **)&l6b, n * 3 * 4));
  B.l6 = l6;
  B.l6b = l6b;
  for (void **p : {&B.xin, &B.w[0], &B.w[1]}) SG_TRY(galloc(G, p, n * 4 * 4));
  B.g = G->fold;
  // sliced-ELLPACK copy of the pattern: rows sorted by length per window,
  // slice sizes, their offsets, then columns and CSR sources per entry
  const int64_t nwin = ((int64_t)g.n + SL_SIGMA - 1) / SL_SIGMA;
  const int64_t nslice = nwin * (SL_SIGMA / SL_W);
  SG_REQUIRE(nslice < (int64_t)1 << 30, "mpnn: %lld slices", (long long)nslice);
  uint32_t *row = nullptr, *ptr = nullptr, *col = nullptr, *src = nullptr;
  SG_TRY(galloc(G, (void **)&row, (size_t)nslice * SL_W * 4));
  SG_TRY(galloc(G, (void **)&ptr, (size_t)(nslice + 1) * 4));
  k_sell_sort<<<(unsigned)nwin, SL_SIGMA, 0, c->stream>>>(g.n, g.rowptr, row);
  {
    Scratch s(c);
    SG_TRY(s.reserve(Scratch::bytes_for(nslice, 4) + scan_scratch_bytes(nslice) + 512));
    uint32_t *cnt = s.alloc<uint32_t>(nslice);
    k_sell_count<<<grid_for(c, nslice, 256, 8), 256, 0, c->stream>>>((int32_t)nslice, g.rowptr,
                                                                     row, cnt);
    SG_CHECK_LAUNCH();
    SG_TRY(exclusive_scan_u32(c, s, cnt, ptr, nslice));
  }
  uint32_t total = 0;
  SG_CHECK_CUDA(cudaMemcpyAsync(&total, ptr + nslice, 4, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  SG_REQUIRE((int64_t)total >= (int64_t)g.nnzb, "mpnn: slice layout holds %u of %lld entries",
             total, (long long)g.nnzb);
  G->sl_total = total;
  SG_TRY(galloc(G, (void **)&col, (size_t)total * 4));
  SG_TRY(galloc(G, (void **)&src, (size_t)total * 4));
  SG_TRY(galloc(G, (void **)&G->ah, (size_t)total * 2));
  SG_TRY(galloc(G, (void **)&G->af, (size_t)total * 4));
  k_sell_fill<<<grid_for(c, nslice * SL_W, 256, 8), 256, 0, c->stream>>>(
      (int32_t)nslice, g.rowptr, g.colidx, row, ptr, col, src);
  SG_CHECK_LAUNCH();
  B.sl.nslice = (int32_t)nslice;
  B.sl.row = row;
  B.sl.ptr = ptr;
  B.sl.col = col;
  B.sl.src = src;
  G->fold_ready = true;
  return graph_refresh(G);
}

// One Horner step on a persistent grid (resident CTAs on every SM, at most
// one warp per slice).
// The Horner steps' grid: one persistent wave (CTAs per SM from the
// occupancy of the plain step), at most one warp per slice.  The last step
// with the end of the application folded in (FIN) runs on the same grid, so
// the solver knows its number of dot partials in advance.
static int horner_grid(GraphH *G, bool half_a, int *out) {
  Ctx *c = G->c;
  static PerDeviceOnce once;
  static int per_sm[SG_MAX_DEVICES][2] = {};
  const int dev = (c->device >= 0 && c->device < SG_MAX_DEVICES) ? c->device : 0;
  SG_TRY(once_per_device(once, dev, [&]() -> int {
    SG_CHECK_CUDA(cudaFuncSetAttribute(k_horner<__half>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)ht_smem_bytes<__half>()));
    SG_CHECK_CUDA(cudaFuncSetAttribute(k_horner<float>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)ht_smem_bytes<float>()));
    SG_CHECK_CUDA(cudaFuncSetAttribute(k_horner<__half, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)ht_smem_bytes<__half>()));
    SG_CHECK_CUDA(cudaFuncSetAttribute(k_horner<float, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)ht_smem_bytes<float>()));
    SG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm[dev][0], k_horner<__half>, HT_WARPS * 32, ht_smem_bytes<__half>()));
    SG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm[dev][1], k_horner<float>, HT_WARPS * 32, ht_smem_bytes<float>()));
    for (int k = 0; k < 2; ++k)
      if (per_sm[dev][k] < 1) per_sm[dev][k] = 1;
    return SG_OK;
  }));
  const int64_t need = ((int64_t)G->fb.sl.nslice + HT_WARPS - 1) / HT_WARPS;
  int64_t grid = (int64_t)c->num_sms * per_sm[dev][half_a ? 0 : 1];
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  *out = (int)grid;
  return SG_OK;
}

static int horner_launch(GraphH *G, cudaStream_t st, const SolveCtl *ctl, int gate, bool half_a,
                         const FoldBufs &B, int d, const void *src, void *dst,
                         const FinArgs *fa = nullptr) {
  Ctx *c = G->c;
  int grid = 1;
  SG_TRY(horner_grid(G, half_a, &grid));
  if (fa) {
    if (half_a)
      k_horner<__half, true><<<(unsigned)grid, HT_WARPS * 32, ht_smem_bytes<__half>(), st>>>(
          ctl, gate, B, d, src, dst, d == 5, c->d_err, *fa);
    else
      k_horner<float, true><<<(unsigned)grid, HT_WARPS * 32, ht_smem_bytes<float>(), st>>>(
          ctl, gate, B, d, src, dst, d == 5, c->d_err, *fa);
  } else if (half_a) {
    k_horner<__half><<<(unsigned)grid, HT_WARPS * 32, ht_smem_bytes<__half>(), st>>>(
        ctl, gate, B, d, src, dst, d == 5, c->d_err);
  } else {
    k_horner<float><<<(unsigned)grid, HT_WARPS * 32, ht_smem_bytes<float>(), st>>>(
        ctl, gate, B, d, src, dst, d == 5, c->d_err);
  }
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// The folded application z = M r (symmetric form): x = L^-1 r (unless the
// iteration's K2 wrote it: xin_ready), the six Horner steps (the first one
// gathers x and applies G_6), z = L^-T w_0.  part (nullable): dot partials of
// the final pass (grid np blocks); want_rr / want_zq select its slices.  The
// FP16 evaluation (half_a) stores x and the Horner sums in block floating
// point, the FP32 one as float4.
static int fold_apply(GraphH *G, cudaStream_t st, const SolveCtl *ctl, int gate, bool half_a,
                      const float *r, float *z, const float *q, double *part, int np, int want_rr,
                      int want_zq, bool xin_ready, bool fused = false,
                      SolveCtl *decide_ctl = nullptr, int par = 0) {
  Ctx *c = G->c;
  Graph &g = G->g;
  FoldBufs B = G->fb;
  B.a = half_a ? (const void *)G->ah : (const void *)G->af;
  // k_lrn_finish moves r, q and z as float4
  SG_REQUIRE(((uintptr_t)r | (uintptr_t)z | (uintptr_t)q) % 16 == 0,
             "mpnn: r, z and q must be 16-byte aligned");
  if (!xin_ready) {
    if (half_a)
      k_lrn_xin<true><<<grid_for(c, g.n, 256, 8), 256, 0, st>>>(g.n, B.l6b, r, B.xin);
    else
      k_lrn_xin<false><<<grid_for(c, g.n, 256, 8), 256, 0, st>>>(g.n, B.l6, r, B.xin);
    SG_CHECK_LAUNCH();
  }
  // step 5 gathers x; step d < 5 reads w[(5 - d) & 1]; step d writes
  // w[(6 - d) & 1] (w_0 in w[0]).  fused: step 0 ends the application itself
  // (z and the dot partials, np of them: the steps' grid)
  for (int d = 5; d >= 0; --d) {
    FinArgs fa;
    if (fused && d == 0) {
      int hg = 0;
      SG_TRY(horner_grid(G, half_a, &hg));
      SG_REQUIRE(!part || np == hg, "mpnn: %d dot partials asked of a %d-CTA last step", np, hg);
      fa.r = r;
      fa.q = q;
      fa.z = z;
      fa.part = part;
      fa.want_rr = want_rr;
      fa.want_zq = want_zq;
      if (decide_ctl && part && want_rr && want_zq) {
        fa.ctl = decide_ctl;
        fa.decide = 1;
        fa.par = par;
      }
    }
    SG_TRY(horner_launch(G, st, ctl, gate, half_a, B, d, d == 5 ? B.xin : B.w[(5 - d) & 1],
                         B.w[(6 - d) & 1], (fused && d == 0) ? &fa : nullptr));
  }
  if (fused) return SG_OK;
  // z = L^-T w_0 and the dots, in vertex order; one dot partial per block:
  // np of them when asked
  const int g0 = part ? np : finish_grid(c, B.sl.nslice);
  if (half_a)
    k_lrn_finish<true><<<g0, LG_T, 0, st>>>(ctl, gate, g.n, B.l6b, B.xin, B.w[0], r, q, z, part,
                                            want_rr, want_zq);
  else
    k_lrn_finish<false><<<g0, LG_T, 0, st>>>(ctl, gate, g.n, B.l6, B.xin, B.w[0], r, q, z, part,
                                             want_rr, want_zq);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// Polynomial coefficients of a parameter set (one small kernel).
static int fold_params(GraphH *G, cudaStream_t st, const float *prm) {
  k_fold<<<1, 256, 0, st>>>(prm, G->fold);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

static int ensure_train(GraphH *G) {
  if (G->train_ready) return SG_OK;
  Graph &g = G->g;
  const size_t n = (size_t)g.n;
  for (float **p : {&g.g1, &g.g2, &g.g3, &g.dg1, &g.dg2, &g.dg3, &g.dh1a, &g.dh2a})
    SG_TRY(galloc(G, (void **)p, n * H * 4));
  for (float **p : {&g.dm2, &g.dm3, &g.dq2, &g.dq3}) SG_TRY(galloc(G, (void **)p, n * K * 4));
  g.gpart_chunks = (int)((n + OUTER_CHUNK - 1) / OUTER_CHUNK);
  SG_TRY(galloc(G, (void **)&g.gpart, (size_t)g.gpart_chunks * H * H * 4));
  SG_TRY(galloc(G, (void **)&g.ld, n * 3 * 4));
  SG_TRY(galloc(G, (void **)&g.lq, n * 3 * 4));
  G->train_ready = true;
  return SG_OK;
}

// The network's layers F2..F4 on input s (already staged): out = s + Wout h3.
// wx/tout: the extra projection of the transposed network's pass.
static int layers(GraphH *G, cudaStream_t st, const SolveCtl *ctl, int gate, const float *prm,
                  const float *s, float *out, bool train, const float *wx = nullptr,
                  float *tout = nullptr) {
  Ctx *c = G->c;
  Graph &g = G->g;
  const int gv = grid_for(c, g.n, 256, 8);
  const int lin = g.lin | (g.sym ? 2 : 0);
  k_f2<<<gv, 256, 0, st>>>(ctl, gate, lin, g.n, g.rowptr, g.colidx, g.a, prm, s, g.m1, g.q2,
                           train ? g.g1 : nullptr);
  SG_CHECK_LAUNCH();
  // one wave of resident CTAs (a partial second wave would run the last
  // CTAs' tiles at a fraction of the occupancy)
  static PerDeviceOnce occ_once;
  static int per_sm_dev[SG_MAX_DEVICES] = {};
  const int dev = (c->device >= 0 && c->device < SG_MAX_DEVICES) ? c->device : 0;
  SG_TRY(once_per_device(occ_once, dev, [&]() -> int {
    int a3 = 0, a4 = 0;
    SG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a3, k_f3, TC_WARPS * 32,
                                                                tc_smem_bytes()));
    SG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a4, k_f4, TC_WARPS * 32,
                                                                tc_smem_bytes()));
    per_sm_dev[dev] = a3 < a4 ? a3 : a4;
    if (per_sm_dev[dev] < 1) per_sm_dev[dev] = 1;
    return SG_OK;
  }));
  const int per_sm = per_sm_dev[dev];
  const int64_t ntile = ((int64_t)g.n + 15) / 16;
  int gt = (int)((ntile + TC_WARPS - 1) / TC_WARPS);
  const int cap = c->num_sms * per_sm;
  if (gt > cap) gt = cap;
  k_f3<<<gt, TC_WARPS * 32, tc_smem_bytes(), st>>>(ctl, gate, lin, g.n, g.rowptr, g.colidx, g.a, prm, s,
                                                   g.m1, g.q2, g.m2, g.q3, train ? g.g2 : nullptr);
  SG_CHECK_LAUNCH();
  k_f4<<<gt, TC_WARPS * 32, tc_smem_bytes(), st>>>(ctl, gate, lin, g.n, g.rowptr, g.colidx, g.a, prm, s,
                                                   g.m1, g.m2, g.q3, g.m3, out, train ? g.g3 : nullptr,
                                                   wx, tout);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// Forward on stream st; ctl may be null (standalone) or the solver control.
// Symmetric form: y = (I + N) L^-1 r on this graph's buffers (training
// activations kept when train), then the transposed network on the twin's
// buffers, then z = L^-T (wp + sum_u a_vu t_u).
static int forward(GraphH *G, cudaStream_t st, const SolveCtl *ctl, int gate, const float *prm,
                   const float *r, float *z, bool train) {
  Ctx *c = G->c;
  Graph &g = G->g;
  const int gv = grid_for(c, g.n, 256, 8);
  if (!g.sym) {
    k_f1<<<gv, 256, 0, st>>>(ctl, gate, g.n, g.dinv, r, g.s, z);
    SG_CHECK_LAUNCH();
    return layers(G, st, ctl, gate, prm, g.s, z, train);
  }
  k_f1<<<gv, 256, 0, st>>>(ctl, gate, g.n, g.linv, r, g.s, nullptr);
  SG_CHECK_LAUNCH();
  SG_TRY(layers(G, st, ctl, gate, prm, g.s, g.y, train));
  k_transpose_params<<<(NPARAM + 255) / 256, 256, 0, st>>>(prm, g.prmT);
  SG_CHECK_LAUNCH();
  SG_TRY(layers(G->twin, st, ctl, gate, g.prmT, g.y, g.wp, false, prm, g.t));
  k_sym_out<<<gv, 256, 0, st>>>(ctl, gate, g.n, g.rowptr, g.colidx, g.a, g.linv, g.wp, g.t, g.s, z);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

static int outer(GraphH *G, const float *X, int O, const float *Y, int I, int ytr, float *dst) {
  Ctx *c = G->c;
  Graph &g = G->g;
  k_outer<<<g.gpart_chunks, 256, 0, c->stream>>>(g.n, X, O, Y, I, ytr, g.gpart);
  SG_CHECK_LAUNCH();
  k_outer_sum<<<(O * I + 255) / 256, 256, 0, c->stream>>>(g.gpart, g.gpart_chunks, O * I, dst);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

static int backward_net(GraphH *G, const float *prm, const float *dz, float *grad);

// Weight gradient of <dz, M r>.  Symmetric form: the network's gradient at
// input L^-1 r with cotangent (I + N) L^-1 dz, plus its gradient at input
// L^-1 dz with cotangent y = (I + N) L^-1 r; the second forward runs on the
// twin's buffers so the first pass's activations survive.
static int backward(GraphH *G, const float *prm, const float *dz, float *grad) {
  Graph &g = G->g;
  if (!g.sym) return backward_net(G, prm, dz, grad);
  GraphH *T = G->twin;
  Ctx *c = G->c;
  SG_TRY(ensure_train(T));
  const int gv = grid_for(c, g.n, 256, 8);
  k_f1<<<gv, 256, 0, c->stream>>>(nullptr, 0, g.n, g.linv, dz, T->g.s, nullptr);
  SG_CHECK_LAUNCH();
  SG_TRY(layers(T, c->stream, nullptr, 0, prm, T->g.s, T->g.y, true));
  SG_TRY(backward_net(G, prm, T->g.y, grad));
  SG_TRY(backward_net(T, prm, g.y, g.gtmp));
  k_add_f<<<(NPARAM + 255) / 256, 256, 0, c->stream>>>(NPARAM, grad, g.gtmp);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

static int backward_net(GraphH *G, const float *prm, const float *dz, float *grad) {
  Ctx *c = G->c;
  Graph &g = G->g;
  SG_TRY(ensure_train(G));
  const int gw = grid_for(c, (int64_t)g.n * 32, 256, 8);
  cudaStream_t st = c->stream;
  k_b1<<<gw, 256, 0, st>>>(g.n, g.lin, prm, dz, g.g3, g.dg3, g.dm3, g.dh2a);
  SG_CHECK_LAUNCH();
  k_bmid<<<gw, 256, 0, st>>>(g.n, g.lin, g.rowptr, g.colidx, g.a, prm, O_P3, O_W2M, O_W2H, g.dm3, g.dh2a,
                             g.g2, g.dq3, g.dg2, g.dm2, g.dh1a);
  SG_CHECK_LAUNCH();
  k_bmid<<<gw, 256, 0, st>>>(g.n, g.lin, g.rowptr, g.colidx, g.a, prm, O_P2, 0, 0, g.dm2, g.dh1a, g.g1,
                             g.dq2, g.dg1, nullptr, nullptr);
  SG_CHECK_LAUNCH();
  // weight gradients; h = act(g) (relu, or identity in the linear variant)
  // the tensor-core operand is bf16(h), or ~h itself with split activations
  const int A_ = g.lin ? 0 : 1, AB = g.sym ? 0 : (g.lin ? 4 : 2);
  SG_TRY(outer(G, dz, 3, g.g3, H, A_, grad + O_WOUT));
  SG_TRY(outer(G, g.dg3, H, g.g2, H, AB, grad + O_W3H));
  SG_TRY(outer(G, g.dg3, H, g.m3, K, 0, grad + O_W3M));
  SG_TRY(outer(G, g.dq3, K, g.g2, H, A_, grad + O_P3));
  SG_TRY(outer(G, g.dg2, H, g.g1, H, AB, grad + O_W2H));
  SG_TRY(outer(G, g.dg2, H, g.m2, K, 0, grad + O_W2M));
  SG_TRY(outer(G, g.dq2, K, g.g1, H, A_, grad + O_P2));
  SG_TRY(outer(G, g.dg1, H, g.s, 3, 0, grad + O_W1S));
  SG_TRY(outer(G, g.dg1, H, g.m1, 3, 0, grad + O_W1M));
  return SG_OK;
}

}  // namespace mpnn

// ---------------------------------------------------------------------------
// solver hooks (SG_PRECOND_LEARNED)
// ---------------------------------------------------------------------------
struct LearnedExt {
  mpnn::GraphH *G = nullptr;
  const float *prm = nullptr;
  int exec = SG_MPNN_EXEC_FOLDED;  // folded (FP16 or FP32 edge weights) or layered
};

static bool folded(const LearnedExt *L) { return L->exec != SG_MPNN_EXEC_LAYERED; }

// K2 of the folded learned iteration (replaces k_cg_update_v4): r update and
// x = L^-1 r; x += alpha p moves to K3.
static int learned_k2(Solver *S, cudaStream_t st, int par) {
  LearnedExt *L = (LearnedExt *)S->ext;
  // the TMA-staged and symmetric-storage K1 leave the p.q total in ctl
  const int pq_fin = (S->tma || S->sym) ? 1 : 0;
  const mpnn::FoldBufs &B = L->G->fb;
  if (L->exec == SG_MPNN_EXEC_FOLDED)
    mpnn::k_lrn_update<true><<<S->P2, RED_T, 0, st>>>(S->ctl, par, S->A.n, S->part1, S->P1,
                                                      pq_fin, (const float *)S->q,
                                                      (float *)S->r, B.l6b, B.xin);
  else
    mpnn::k_lrn_update<false><<<S->P2, RED_T, 0, st>>>(S->ctl, par, S->A.n, S->part1, S->P1,
                                                       pq_fin, (const float *)S->q,
                                                       (float *)S->r, B.l6, B.xin);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

static int learned_prec(Solver *S, cudaStream_t st, int par) {
  LearnedExt *L = (LearnedExt *)S->ext;
  if (folded(L))
    // the last Horner step leaves r.r | r.z | z.q summed and the iteration
    // decided (status, beta) in ctl for K3
    return mpnn::fold_apply(L->G, st, S->ctl, 1, L->exec == SG_MPNN_EXEC_FOLDED,
                            (const float *)S->r, (float *)S->z, (const float *)S->q, S->part2,
                            S->np2_ext, 1, 1, true, true, S->ctl, par);
  SG_TRY(mpnn::forward(L->G, st, S->ctl, 1, L->prm, (const float *)S->r, (float *)S->z, false));
  mpnn::k_rz_zq<<<S->P2, RED_T, 0, st>>>(S->ctl, S->len, (const float *)S->r, (const float *)S->z,
                                         (const float *)S->q, S->part2);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// Set-up / restart: z = M(r) with the network (or Jacobi after a fallback),
// partials of r.z into part3 (P2 blocks).
__global__ void __launch_bounds__(RED_T) k_rz_only(int64_t len, const float *r, const float *z,
                                                   double *part) {
  __shared__ double sh[33];
  double rz = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    rz += (double)r[i] * (double)z[i];
  const double t = block_sum(rz, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

static int learned_apply(Solver *S, cudaStream_t st) {
  LearnedExt *L = (LearnedExt *)S->ext;
  // the control block's fallback flag also governs restarts
  if (folded(L)) {
    // the parameters may have changed since the last solve: fold them again
    SG_TRY(mpnn::fold_params(L->G, st, L->prm));
    return mpnn::fold_apply(L->G, st, S->ctl, 0, L->exec == SG_MPNN_EXEC_FOLDED,
                            (const float *)S->r, (float *)S->z, nullptr, S->part3, S->P2, 0, 0,
                            false);
  }
  SG_TRY(mpnn::forward(L->G, st, S->ctl, 0, L->prm, (const float *)S->r, (float *)S->z, false));
  k_rz_only<<<S->P2, RED_T, 0, st>>>(S->len, (const float *)S->r, (const float *)S->z, S->part3);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

static void learned_free(Solver *S) {
  LearnedExt *L = (LearnedExt *)S->ext;
  if (!L) return;
  mpnn::graph_free(L->G);
  delete L;
  S->ext = nullptr;
}

// solver_init calls learned_setup on the creating thread: the settings pass
// through thread-local slots, so solvers may be created concurrently
static thread_local const float *g_pending_params = nullptr;
static thread_local int g_pending_form = 0;
static thread_local int g_pending_exec = 0;
static int learned_setup(Solver *S) {
  LearnedExt *L = new LearnedExt();
  S->ext = L;
  S->ext_free = learned_free;
  L->prm = g_pending_params;
  L->G = new mpnn::GraphH();
  SG_TRY(mpnn::graph_init(S->c, &S->A, L->G));
  SG_TRY(mpnn::set_sym(L->G, g_pending_form == SG_MPNN_SYM));
  L->G->g.lin = g_pending_form != SG_MPNN_RELU;
  // the folded evaluation serves the symmetric form; the others run layered
  L->exec = g_pending_form == SG_MPNN_SYM ? g_pending_exec : SG_MPNN_EXEC_LAYERED;
  S->ext_prec = learned_prec;
  S->ext_prec_apply = learned_apply;
  S->flexible = 1;
  if (folded(L)) {
    SG_TRY(mpnn::ensure_folded(L->G));
    S->ext_k2 = learned_k2;
    S->k3_xupd = 1;
    S->ext_decides = 1;
    // the last Horner step, with the end of the application folded in,
    // runs on the steps' grid and leaves that many partials per dot for K3
    int g0 = 0;
    SG_TRY(mpnn::horner_grid(L->G, L->exec == SG_MPNN_EXEC_FOLDED, &g0));
    const int np = S->P1 > S->P2 ? S->P1 : S->P2;
    if (g0 > np) {
      void *p2 = nullptr;
      SG_CHECK_CUDA(cudaMalloc(&p2, (size_t)g0 * 3 * 8));
      S->allocs.push_back(p2);
      S->part2 = (double *)p2;
    }
    S->np2_ext = g0;
  }
  return SG_OK;
}

int learned_refresh(Solver *S) {
  LearnedExt *L = (LearnedExt *)S->ext;
  return L ? mpnn::graph_refresh(L->G) : SG_OK;
}

int learned_solver_init(Ctx *c, const sg_matrix *A, const sg_solve_opts *o, const float *params,
                        Solver *S) {
  g_pending_params = params;
  g_pending_form = o->learned_form;
  g_pending_exec = o->learned_exec;
  int rc = solver_init(c, A, o, S, learned_setup);
  g_pending_params = nullptr;
  return rc;
}

}  // namespace sg

using namespace sg;

extern "C" {

int sg_mpnn_nparams(void) { return mpnn::NPARAM; }

int sg_mpnn_graph_create(sg_ctx *h, const sg_matrix *A, sg_mpnn_graph **out) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && A && out, "sg_mpnn_graph_create: null argument");
  mpnn::GraphH *G = new mpnn::GraphH();
  int rc = mpnn::graph_init(c, A, G);
  if (rc != SG_OK) {
    mpnn::graph_free(G);
    return rc;
  }
  ctx_retain(c);
  *out = reinterpret_cast<sg_mpnn_graph *>(G);
  return SG_OK;
}

int sg_mpnn_graph_set_form(sg_mpnn_graph *hg, int form) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  SG_REQUIRE(G, "sg_mpnn_graph_set_form: null graph");
  SG_REQUIRE(form >= SG_MPNN_RELU && form <= SG_MPNN_SYM, "sg_mpnn_graph_set_form: form %d", form);
  SG_TRY(mpnn::set_sym(G, form == SG_MPNN_SYM));
  G->g.lin = form != SG_MPNN_RELU;
  return SG_OK;
}

int sg_mpnn_graph_refresh(sg_mpnn_graph *hg) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  SG_REQUIRE(G, "sg_mpnn_graph_refresh: null graph");
  return mpnn::graph_refresh(G);
}

int sg_mpnn_graph_destroy(sg_mpnn_graph *hg) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  if (!G) return SG_OK;
  cudaStreamSynchronize(G->c->stream);
  Ctx *c = G->c;
  mpnn::graph_free(G);
  ctx_release(c);
  return SG_OK;
}

int sg_mpnn_graph_set_exec(sg_mpnn_graph *hg, int exec) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  SG_REQUIRE(G, "sg_mpnn_graph_set_exec: null graph");
  SG_REQUIRE(exec >= SG_MPNN_EXEC_FOLDED && exec <= SG_MPNN_EXEC_FOLDED_F32,
             "sg_mpnn_graph_set_exec: mode %d", exec);
  SG_REQUIRE(exec == SG_MPNN_EXEC_LAYERED || G->g.sym,
             "sg_mpnn_graph_set_exec: the folded evaluation needs the symmetric form");
  if (exec != SG_MPNN_EXEC_LAYERED) SG_TRY(mpnn::ensure_folded(G));
  G->exec = exec;
  return SG_OK;
}

int sg_mpnn_fold_step(sg_mpnn_graph *hg, int32_t d) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  SG_REQUIRE(G && d >= 0 && d <= 5, "sg_mpnn_fold_step: bad argument");
  SG_REQUIRE(G->fold_ready && G->exec != SG_MPNN_EXEC_LAYERED,
             "sg_mpnn_fold_step: no folded evaluation on this graph");
  mpnn::FoldBufs B = G->fb;
  const bool half_a = G->exec == SG_MPNN_EXEC_FOLDED;
  B.a = half_a ? (const void *)G->ah : (const void *)G->af;
  return mpnn::horner_launch(G, G->c->stream, nullptr, 0, half_a, B, d,
                             d == 5 ? B.xin : B.w[(5 - d) & 1], B.w[(6 - d) & 1]);
}

int sg_mpnn_forward(sg_mpnn_graph *hg, const float *params, const float *r, float *z, int train) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  SG_REQUIRE(G && params && r && z, "sg_mpnn_forward: null argument");
  if (!train && G->exec != SG_MPNN_EXEC_LAYERED && G->g.sym) {
    SG_TRY(mpnn::fold_params(G, G->c->stream, params));
    return mpnn::fold_apply(G, G->c->stream, nullptr, 0, G->exec == SG_MPNN_EXEC_FOLDED, r, z,
                            nullptr, nullptr, 0, 0, 0, false);
  }
  if (train) SG_TRY(mpnn::ensure_train(G));
  return mpnn::forward(G, G->c->stream, nullptr, 0, params, r, z, train != 0);
}

int sg_mpnn_backward(sg_mpnn_graph *hg, const float *params, const float *dz, float *grad) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  SG_REQUIRE(G && params && dz && grad, "sg_mpnn_backward: null argument");
  SG_REQUIRE(G->train_ready, "sg_mpnn_backward: run sg_mpnn_forward with train=1 first");
  return mpnn::backward(G, params, dz, grad);
}

int sg_mpnn_loss(sg_mpnn_graph *hg, const float *z, const float *e, double eAe, float *dz,
                 double *h_loss) {
  mpnn::GraphH *G = reinterpret_cast<mpnn::GraphH *>(hg);
  DeviceGuard dg_(G ? G->c : nullptr);
  SG_REQUIRE(G && z && e && dz && h_loss && eAe > 0, "sg_mpnn_loss: bad argument");
  SG_REQUIRE(G->g.vdt == SG_F32, "sg_mpnn_loss: the graph's matrix must be FP32");
  SG_TRY(mpnn::ensure_train(G));
  Ctx *c = G->c;
  mpnn::Graph &g = G->g;
  const int64_t len = (int64_t)g.n * 3;
  const int gr = grid_for(c, len, 256, 8);
  mpnn::k_sub<<<gr, 256, 0, c->stream>>>(len, z, e, g.ld);
  SG_CHECK_LAUNCH();
  SG_TRY(bspmv_launch(c, g.n, 3, g.rowptr, g.colidx, g.vdt, g.vals, SG_F32, g.ld, g.lq, 0, g.nnzb));
  double dAd = 0;
  SG_TRY(sg_dot(reinterpret_cast<sg_ctx *>(c), len, SG_F32, g.ld, g.lq, &dAd));
  *h_loss = dAd / eAe;
  mpnn::k_scale<<<gr, 256, 0, c->stream>>>(len, g.lq, (float)(2.0 / eAe), dz);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

int sg_mpnn_adam(sg_ctx *h, float *params, const float *grad, float *m, float *v, int step,
                 float lr, float beta1, float beta2, float eps) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && params && grad && m && v && step >= 1, "sg_mpnn_adam: bad argument");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  mpnn::k_adam<<<(mpnn::NPARAM + 255) / 256, 256, 0, c->stream>>>(mpnn::NPARAM, params, grad, m, v,
                                                                  lr, beta1, beta2, eps, c1, c2);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // extern "C"
