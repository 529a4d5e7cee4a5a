// Evaluation of the symmetric factorized form of the learned
// preconditioner (see sg_mpnn.cuh) as a matrix polynomial.
//
// The symmetric form uses the linear network N.  With identity activations
// every hidden layer of width 64 is a fixed linear function of the inputs
// and messages that precede it, and every per-vertex linear map commutes
// with the edge-weight aggregation Aw (the same map at every vertex), so
// the network is exactly a cubic polynomial in Aw with 3x3 coefficients
// and the preconditioner a degree-6 one:
//
//   M = L^-T [ sum_{d=0..6} Aw^d (x) G_d ] L^-1,   G_d symmetric 3x3.
//
// k_fold computes G_0..G_6 once per parameter set, in FP64, from the same
// bf16-rounded W2h/W3h the tensor-core layers use.  One application is then
// x = L^-1 r and w_6 = G_6 x (fused into the iteration's r update), six
// Horner steps w_d = G_d x + Aw w_{d+1}, each a gather of a 3-wide vector
// over the matrix pattern, and z = L^-T w_0 with the iteration's dot
// products fused into the last step -- instead of twelve 64x64 tensor-core
// products per 16-vertex tile and seven gather passes of up to 8-wide
// messages.  The operator is the one the layered kernels evaluate (their
// split-bf16 activations carry the hidden layers to about 2^-16); tests
// compare the two and the oracle's restatement.
//
// Layout: x and the Horner sums are [n][4] (float4 per vertex); the passes
// read the pattern and the edge weights (FP16 by default, FP32 on request)
// from a sliced-ELLPACK copy with one lane per row (SellGraph below).
#pragma once
#include <cuda_fp16.h>

#include "sg_mpnn.cuh"
#include "sg_solver_kernels.cuh"

namespace sg {
namespace mpnn {

// Intermediate folded matrices (FP64, row-major): C2 [8][6] | C3 [8][14] |
// C4 [3][22].  C4's column blocks: x 0..2, m1 3..5, m2 6..13, m3 14..21;
// C3's: x 0..2, m1 3..5, m2 6..13; C2's: x 0..2, m1 3..5.
constexpr int FO_C2 = 0, FO_C3 = 48, FO_C4 = 48 + 112, NFOLD = 48 + 112 + 66;

// The network as a polynomial: the per-vertex maps commute with the
// aggregation ((I (x) C)(Aw (x) I) = Aw (x) C), so
//   N = sum_{k=0..3} Aw^k (x) B_k,       B_0 = C4x,
//   B_1 = C4m1 + C4m2 C2x + C4m3 C3x,   B_2 = C4m2 C2m1 + C4m3 (C3m1 + C3m2 C2x),
//   B_3 = C4m3 C3m2 C2m1,
// and with B'_0 = I + B_0, B'_k = B_k,
//   (I+N)^T (I+N) = sum_{d=0..6} Aw^d (x) G_d,   G_d = sum_{j+k=d} B'_j^T B'_k,
// each G_d symmetric.  k_fold writes G_0..G_6 (FP32, 9 values each,
// symmetrised in FP64 before rounding).  One block of 256 threads.
__global__ void __launch_bounds__(256) k_fold(const float *__restrict__ prm,
                                              float *__restrict__ gout) {
  __shared__ double E1[H * 6], F2[H * 14], F3[H * 22], Cf[NFOLD];
  const int t = threadIdx.x;
  for (int i = t; i < H * 6; i += 256) {
    const int h = i / 6, c = i % 6;
    E1[i] = c < 3 ? prm[O_W1S + h * 3 + c] : prm[O_W1M + h * 3 + c - 3];
  }
  __syncthreads();
  for (int i = t; i < H * 14; i += 256) {
    const int r = i / 14, c = i % 14;
    double s = 0.0;
    if (c < 6)
      for (int h = 0; h < H; ++h) s += (double)bf16r(prm[O_W2H + r * H + h]) * E1[h * 6 + c];
    else
      s = prm[O_W2M + r * K + c - 6];
    F2[i] = s;
  }
  __syncthreads();
  for (int i = t; i < H * 22; i += 256) {
    const int r = i / 22, c = i % 22;
    double s = 0.0;
    if (c < 14)
      for (int h = 0; h < H; ++h) s += (double)bf16r(prm[O_W3H + r * H + h]) * F2[h * 14 + c];
    else
      s = prm[O_W3M + r * K + c - 14];
    F3[i] = s;
  }
  __syncthreads();
  for (int i = t; i < NFOLD; i += 256) {
    double s = 0.0;
    if (i < FO_C3) {
      const int j = i / 6, c = i % 6;
      for (int h = 0; h < H; ++h) s += (double)prm[O_P2 + j * H + h] * E1[h * 6 + c];
    } else if (i < FO_C4) {
      const int j = (i - FO_C3) / 14, c = (i - FO_C3) % 14;
      for (int h = 0; h < H; ++h) s += (double)prm[O_P3 + j * H + h] * F2[h * 14 + c];
    } else {
      const int k = (i - FO_C4) / 22, c = (i - FO_C4) % 22;
      for (int h = 0; h < H; ++h) s += (double)prm[O_WOUT + k * H + h] * F3[h * 22 + c];
    }
    Cf[i] = s;
  }
  __syncthreads();
  if (t != 0) return;
  // accessors: C2[j][c], C3[j][c], C4[k][c]
  auto c2 = [&](int j, int c) { return Cf[FO_C2 + j * 6 + c]; };
  auto c3 = [&](int j, int c) { return Cf[FO_C3 + j * 14 + c]; };
  auto c4 = [&](int k, int c) { return Cf[FO_C4 + k * 22 + c]; };
  double Bp[4][9];
  for (int k = 0; k < 3; ++k)
    for (int l = 0; l < 3; ++l) {
      // (C3m2 C2x)[i][l] and (C3m2 C2m1)[i][l] for i < 8 enter B_2, B_3
      double b1 = c4(k, 3 + l), b2 = 0.0, b3 = 0.0;
      for (int j = 0; j < 8; ++j) {
        b1 += c4(k, 6 + j) * c2(j, l) + c4(k, 14 + j) * c3(j, l);
        b2 += c4(k, 6 + j) * c2(j, 3 + l);
        double t2 = c3(j, 3 + l), t3 = 0.0;
        for (int i = 0; i < 8; ++i) {
          t2 += c3(j, 6 + i) * c2(i, l);
          t3 += c3(j, 6 + i) * c2(i, 3 + l);
        }
        b2 += c4(k, 14 + j) * t2;
        b3 += c4(k, 14 + j) * t3;
      }
      Bp[0][k * 3 + l] = (k == l ? 1.0 : 0.0) + c4(k, l);
      Bp[1][k * 3 + l] = b1;
      Bp[2][k * 3 + l] = b2;
      Bp[3][k * 3 + l] = b3;
    }
  for (int d = 0; d < 7; ++d) {
    double Gd[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < 4; ++j) {
      const int k = d - j;
      if (k < 0 || k > 3) continue;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          for (int m = 0; m < 3; ++m) Gd[a * 3 + b] += Bp[j][m * 3 + a] * Bp[k][m * 3 + b];
    }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        gout[d * 9 + a * 3 + b] = (float)(0.5 * (Gd[a * 3 + b] + Gd[b * 3 + a]));
  }
}

// Packed lower-triangular L_v^-1 (l00, l10, l11, l20, l21, l22) from the
// 9-value form k_chol_inv writes.
__global__ void k_pack_linv(int32_t n, const float *__restrict__ linv, float *__restrict__ l6) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const float *L = linv + v * 9;
    float *o = l6 + v * 6;
    o[0] = L[0]; o[1] = L[3]; o[2] = L[4]; o[3] = L[6]; o[4] = L[7]; o[5] = L[8];
  }
}

__device__ __forceinline__ float ldw(const float *a, uint32_t q) { return __ldg(a + q); }
__device__ __forceinline__ float ldw(const __half *a, uint32_t q) {
  return __half2float(__ldg(a + q));
}

// ---------------------------------------------------------------------------
// Sliced-ELLPACK copy of the pattern for the Horner passes
// ---------------------------------------------------------------------------
// A Horner pass gathers one 3-wide vector per edge.  With a row reduced by
// several lanes (CSR order) one warp instruction touches the cache lines of
// up to 32 unrelated neighbours plus 8 rows' worth of index and weight
// segments, and the pass runs at the L1's wavefront rate, not at HBM speed.
// The passes therefore read the pattern as SELL-32-128: rows are sorted by
// length inside windows of SL_SIGMA rows (rows of one length stay in their
// order), every run of 32 sorted rows is a slice that one warp processes
// with one lane per row, and the slice's entries are stored entry-major
// (entry k of lane l at ptr[s] + 32 k + l), so each load of indices or
// weights is one contiguous 128 / 64 byte segment and each gather
// instruction reads entry k of 32 rows that are close in the ordering.
// Slices are as long as their longest row; the shorter rows are padded with
// weight 0 and a valid column.  Built once per pattern; the weights are
// copied into slice order at every refresh.
constexpr int SL_W = 32;          // rows per slice: one warp, one lane each
constexpr int SL_SIGMA = 128;     // rows per sorting window
constexpr int SL_U = 4;           // entries per round of a Horner pass
constexpr uint32_t SL_NONE = 0xffffffffu;
constexpr int LG_T = 256;         // threads per CTA of the Horner passes
constexpr int NPOLY = 7;          // polynomial degree 6

struct SellGraph {
  int32_t nslice = 0;
  const uint32_t *row = nullptr;  // [nslice*32] row of each slice lane, SL_NONE past n
  const uint32_t *ptr = nullptr;  // [nslice+1] first entry of each slice
  const uint32_t *col = nullptr;  // [ptr[nslice]] column of each entry
  const uint32_t *src = nullptr;  // [ptr[nslice]] CSR entry of each entry, SL_NONE = padding
};

// Rows of each window of SL_SIGMA sorted by decreasing length (stable).
// One block of SL_SIGMA threads per window.
__global__ void __launch_bounds__(SL_SIGMA) k_sell_sort(int32_t n, const uint32_t *__restrict__ rowptr,
                                                        uint32_t *__restrict__ row) {
  __shared__ int len[SL_SIGMA];
  const int64_t base = (int64_t)blockIdx.x * SL_SIGMA;
  const int i = threadIdx.x;
  const int64_t v = base + i;
  len[i] = v < n ? (int)(rowptr[v + 1] - rowptr[v]) : -1;
  __syncthreads();
  const int li = len[i];
  int rank = 0;
  for (int j = 0; j < SL_SIGMA; ++j) {
    const int lj = len[j];
    rank += (lj > li) || (lj == li && j < i);
  }
  row[base + rank] = v < n ? (uint32_t)v : SL_NONE;
}

// Entries of each slice: 32 x its longest row.
__global__ void k_sell_count(int32_t nslice, const uint32_t *__restrict__ rowptr,
                             const uint32_t *__restrict__ row, uint32_t *__restrict__ cnt) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nslice;
       s += (int64_t)gridDim.x * blockDim.x) {
    uint32_t m = 0;
    for (int l = 0; l < SL_W; ++l) {
      const uint32_t v = row[s * SL_W + l];
      if (v != SL_NONE) {
        const uint32_t len = rowptr[v + 1] - rowptr[v];
        m = len > m ? len : m;
      }
    }
    cnt[s] = m * SL_W;
  }
}

// Columns and CSR sources of every slice entry; one thread per slice lane.
__global__ void k_sell_fill(int32_t nslice, const uint32_t *__restrict__ rowptr,
                            const uint32_t *__restrict__ colidx, const uint32_t *__restrict__ row,
                            const uint32_t *__restrict__ ptr, uint32_t *__restrict__ col,
                            uint32_t *__restrict__ src) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)nslice * SL_W;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = t / SL_W;
    const int l = (int)(t % SL_W);
    const uint32_t v = row[t];
    const uint32_t b = ptr[s], len = (ptr[s + 1] - b) / SL_W;
    const uint32_t lo = v != SL_NONE ? rowptr[v] : 0u;
    const uint32_t rl = v != SL_NONE ? rowptr[v + 1] - lo : 0u;
    for (uint32_t k = 0; k < len; ++k) {
      const size_t e = (size_t)b + (size_t)k * SL_W + l;
      if (k < rl) {
        col[e] = colidx[lo + k];
        src[e] = lo + k;
      } else {
        col[e] = v != SL_NONE ? v : 0u;
        src[e] = SL_NONE;
      }
    }
  }
}

// Edge weights in slice order (FP16 for the default passes, FP32 for the
// FP32-weight variant); padding entries get 0.
__device__ __forceinline__ void stw(float *o, float w) { *o = w; }
__device__ __forceinline__ void stw(__half *o, float w) { *o = __float2half_rn(w); }
template <typename AT>
__global__ void k_sell_weights(int64_t total, const uint32_t *__restrict__ src,
                               const float *__restrict__ a, AT *__restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t q = src[e];
    stw(out + e, q != SL_NONE ? a[q] : 0.f);
  }
}

// Blocks of a Horner pass over `nslice` slices (also the number of dot
// partials the last pass leaves).
inline int horner_grid(const Ctx *c, int32_t nslice) {
  return grid_for(c, (int64_t)nslice * SL_W, LG_T, 8);
}

// Buffers of one folded application.
struct FoldBufs {
  SellGraph sl;
  const void *a;      // FP32 or FP16 edge weights in slice order
  const float *g;     // the 7 symmetric 3x3 coefficients G_0..G_6, row-major
  const float *l6;    // packed L^-1 [n][6]
  float *xin;         // x = L^-1 r   [n][4]
  float *w[2];        // Horner partial sums, ping-pong [n][4]
};


// One Horner step w_d = G_d x + Aw w_{d+1} (d = 5 .. 0).  A warp takes one
// slice (a lane per row) per step; the entry loop runs to the slice's
// length, the same for every lane, so all lanes reach the shuffles of the
// block sums.  ctl (nullable) gates on the solve status (gate) and, after a
// fallback to block Jacobi, skips the polynomial.  LAST (d = 0):
// z = L^-T w_0 (z = L^-T x = D^-1 r after a fallback) and the dot partials
// of the new z when part != null: r.r at part[0 .. np), r.z at
// part[np .. 2np), z.q at part[2np .. 3np) (np = gridDim.x) when want_rr /
// want_zq, else r.z alone at part[0 .. np).
template <typename AT, bool LAST>
__global__ void __launch_bounds__(LG_T) k_horner(const SolveCtl *ctl, int gate, int32_t n,
                                                 FoldBufs B, int d, const float *__restrict__ src,
                                                 float *__restrict__ dst,
                                                 const float *__restrict__ r,
                                                 const float *__restrict__ q,
                                                 float *__restrict__ z, double *__restrict__ part,
                                                 int want_rr, int want_zq) {
  __shared__ float G[9];
  __shared__ double sh[33];
  if (ctl && gate && ctl->status != ST_RUNNING) return;
  const bool fb = ctl && ctl->fallback;
  if (fb && !LAST) return;
  if (threadIdx.x < 9) G[threadIdx.x] = B.g[d * 9 + threadIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t nwarp = (int64_t)gridDim.x * (blockDim.x >> 5);
  const AT *__restrict__ aw = (const AT *)B.a;
  const float4 *__restrict__ s4 = reinterpret_cast<const float4 *>(src);
  DotAcc<float> rr, rz, zq;
  for (int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
       s < B.sl.nslice; s += nwarp) {
    const uint32_t v = __ldg(B.sl.row + s * SL_W + lane);
    float m0 = 0.f, m1 = 0.f, m2 = 0.f;
    if (!fb) {
      const uint32_t b = __ldg(B.sl.ptr + s), e1 = __ldg(B.sl.ptr + s + 1);
      const uint32_t len = (e1 - b) / SL_W;
      const uint32_t *cp = B.sl.col + b + lane;
      const AT *ap = aw + b + lane;
      uint32_t k = 0;
      // U entries per round: their index, weight and vector loads all issue
      // before the accumulation (the last pass keeps 4: it holds more state)
      constexpr int U = LAST ? 4 : SL_U;
      for (; k + U <= len; k += U) {
        uint32_t u[U];
        float wq[U];
        float4 g[U];
#pragma unroll
        for (int j = 0; j < U; ++j) {
          u[j] = __ldg(cp + (k + j) * SL_W);
          wq[j] = ldw(ap, (k + j) * SL_W);
        }
#pragma unroll
        for (int j = 0; j < U; ++j) g[j] = __ldg(s4 + u[j]);
#pragma unroll
        for (int j = 0; j < U; ++j) {
          m0 += wq[j] * g[j].x;
          m1 += wq[j] * g[j].y;
          m2 += wq[j] * g[j].z;
        }
      }
      for (; k < len; ++k) {
        const uint32_t u = __ldg(cp + k * SL_W);
        const float wq = ldw(ap, k * SL_W);
        const float4 g = __ldg(s4 + u);
        m0 += wq * g.x;
        m1 += wq * g.y;
        m2 += wq * g.z;
      }
    }
    if (v == SL_NONE) continue;
    const float4 x4 = *reinterpret_cast<const float4 *>(B.xin + (size_t)v * 4);
    if (!LAST) {
      *reinterpret_cast<float4 *>(dst + (size_t)v * 4) =
          make_float4(m0 + G[0] * x4.x + G[1] * x4.y + G[2] * x4.z,
                      m1 + G[3] * x4.x + G[4] * x4.y + G[5] * x4.z,
                      m2 + G[6] * x4.x + G[7] * x4.y + G[8] * x4.z, 0.f);
    } else {
      float w0 = x4.x, w1 = x4.y, w2 = x4.z;
      if (!fb) {
        w0 = m0 + G[0] * x4.x + G[1] * x4.y + G[2] * x4.z;
        w1 = m1 + G[3] * x4.x + G[4] * x4.y + G[5] * x4.z;
        w2 = m2 + G[6] * x4.x + G[7] * x4.y + G[8] * x4.z;
      }
      // (L^-1)^T w, L^-1 = [[l0,0,0],[l1,l2,0],[l3,l4,l5]]
      const float2 *L2 = reinterpret_cast<const float2 *>(B.l6 + (size_t)v * 6);
      const float2 la = L2[0], lb = L2[1], lc = L2[2];
      const float zk0 = la.x * w0 + la.y * w1 + lb.y * w2;
      const float zk1 = lb.x * w1 + lc.x * w2;
      const float zk2 = lc.y * w2;
      float *zv = z + (size_t)v * 3;
      zv[0] = zk0;
      zv[1] = zk1;
      zv[2] = zk2;
      if (part) {
        const float *rv = r + (size_t)v * 3;
        const float r0 = rv[0], r1 = rv[1], r2 = rv[2];
        if (want_rr) {
          rr.add(r0, r0);
          rr.add(r1, r1);
          rr.add(r2, r2);
        }
        rz.add(r0, zk0);
        rz.add(r1, zk1);
        rz.add(r2, zk2);
        if (want_zq) {
          const float *qv = q + (size_t)v * 3;
          zq.add(zk0, qv[0]);
          zq.add(zk1, qv[1]);
          zq.add(zk2, qv[2]);
        }
      }
    }
  }
  if (!LAST || !part) return;
  const double t1 = block_sum(rz.value(), sh);
  const double t0 = want_rr ? block_sum(rr.value(), sh) : 0.0;
  const double t2 = want_zq ? block_sum(zq.value(), sh) : 0.0;
  if (threadIdx.x == 0) {
    if (want_rr) part[blockIdx.x] = t0;
    part[(want_rr ? gridDim.x : 0) + blockIdx.x] = t1;
    if (want_zq) part[2 * gridDim.x + blockIdx.x] = t2;
  }
}

// x = L^-1 r and w_6 = G_6 x for a fresh r (set-up, restarts and the
// standalone forward).
__global__ void k_lrn_xin(int32_t n, const float *__restrict__ l6, const float *__restrict__ g6,
                          const float *__restrict__ r, float *__restrict__ xin,
                          float *__restrict__ w6) {
  float G[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) G[k] = __ldg(g6 + k);
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const float *L = l6 + v * 6;
    const float r0 = r[v * 3], r1 = r[v * 3 + 1], r2 = r[v * 3 + 2];
    const float x0 = L[0] * r0, x1 = L[1] * r0 + L[2] * r1, x2 = L[3] * r0 + L[4] * r1 + L[5] * r2;
    *reinterpret_cast<float4 *>(xin + v * 4) = make_float4(x0, x1, x2, 0.f);
    *reinterpret_cast<float4 *>(w6 + v * 4) =
        make_float4(G[0] * x0 + G[1] * x1 + G[2] * x2, G[3] * x0 + G[4] * x1 + G[5] * x2,
                    G[6] * x0 + G[7] * x1 + G[8] * x2, 0.f);
  }
}

// K2 of the learned iteration: alpha = r.z / p.q; r -= alpha q; x = L^-1 r;
// w_6 = G_6 x.  x += alpha p is left to K3 (k_cg_direction_v4 with xupd),
// which decides the iteration from the partials the last Horner step
// leaves.  A thread takes 4 vertices (three float4 of r and q, six of
// L^-1, four each of x and w_6); the last n % 4 vertices go to thread 0 of
// the last CTA.
__global__ void __launch_bounds__(RED_T) k_lrn_update(SolveCtl *ctl, int par, int32_t n,
                                                      const double *__restrict__ part_in,
                                                      int np1, int pq_fin,
                                                      const float *__restrict__ q,
                                                      float *__restrict__ r,
                                                      const float *__restrict__ l6,
                                                      const float *__restrict__ g6,
                                                      float *__restrict__ xin,
                                                      float *__restrict__ w6) {
  __shared__ double sh[33];
  if (ctl->status != ST_RUNNING) return;
  const double pq = pq_fin ? ctl->pq_tot : sum_parts(part_in, np1, sh);
  if (!(pq > 0.0) || !isfinite(pq)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
    return;
  }
  const double alpha = ctl->rz[par] / pq;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->last_alpha = alpha;
  const float a = (float)alpha;
  float G[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) G[k] = __ldg(g6 + k);
  const int64_t nu = n / 4;
  const float4 *q4 = reinterpret_cast<const float4 *>(q);
  float4 *r4 = reinterpret_cast<float4 *>(r);
  const float4 *l4 = reinterpret_cast<const float4 *>(l6);
  float4 *x4 = reinterpret_cast<float4 *>(xin);
  float4 *w4 = reinterpret_cast<float4 *>(w6);
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nu;
       u += (int64_t)gridDim.x * blockDim.x) {
    float rv[12], lv[24];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float4 b = q4[u * 3 + k], c = r4[u * 3 + k];
      rv[4 * k] = c.x - a * b.x;
      rv[4 * k + 1] = c.y - a * b.y;
      rv[4 * k + 2] = c.z - a * b.z;
      rv[4 * k + 3] = c.w - a * b.w;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float4 g = l4[u * 6 + k];
      lv[4 * k] = g.x; lv[4 * k + 1] = g.y; lv[4 * k + 2] = g.z; lv[4 * k + 3] = g.w;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
      r4[u * 3 + k] = make_float4(rv[4 * k], rv[4 * k + 1], rv[4 * k + 2], rv[4 * k + 3]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float *L = lv + 6 * j, *R = rv + 3 * j;
      const float x0 = L[0] * R[0], x1 = L[1] * R[0] + L[2] * R[1],
                  x2 = L[3] * R[0] + L[4] * R[1] + L[5] * R[2];
      x4[u * 4 + j] = make_float4(x0, x1, x2, 0.f);
      w4[u * 4 + j] = make_float4(G[0] * x0 + G[1] * x1 + G[2] * x2, G[3] * x0 + G[4] * x1 + G[5] * x2,
                                  G[6] * x0 + G[7] * x1 + G[8] * x2, 0.f);
    }
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    for (int64_t v = nu * 4; v < n; ++v) {
      float R[3];
      for (int k = 0; k < 3; ++k) {
        R[k] = r[v * 3 + k] - a * q[v * 3 + k];
        r[v * 3 + k] = R[k];
      }
      const float *L = l6 + v * 6;
      const float x0 = L[0] * R[0], x1 = L[1] * R[0] + L[2] * R[1],
                  x2 = L[3] * R[0] + L[4] * R[1] + L[5] * R[2];
      *reinterpret_cast<float4 *>(xin + v * 4) = make_float4(x0, x1, x2, 0.f);
      *reinterpret_cast<float4 *>(w6 + v * 4) =
          make_float4(G[0] * x0 + G[1] * x1 + G[2] * x2, G[3] * x0 + G[4] * x1 + G[5] * x2,
                      G[6] * x0 + G[7] * x1 + G[8] * x2, 0.f);
    }
}

}  // namespace mpnn
}  // namespace sg
