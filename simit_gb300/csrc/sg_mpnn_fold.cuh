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
// Layout: x and the Horner sums are [n][4] (float4 per vertex); the edge
// weights a are FP32 or FP16 beside colidx.  A row is reduced by 4 lanes
// (every 4th entry each, then two shuffles).
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

// FP16 copy of the edge weights (the folded passes' default).
__global__ void k_edge_half(int64_t nnzb, const float *__restrict__ a, __half *__restrict__ ah) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnzb;
       q += (int64_t)gridDim.x * blockDim.x)
    ah[q] = __float2half_rn(a[q]);
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

// Weighted sum over the row [lo, hi) of sum_q a[q] src[colidx[q]][0..W) by
// the 4 lanes of a group (sub = lane & 3 takes entries lo+sub, lo+sub+4,
// ...); all loads of 4 entries are issued before their accumulation.  On
// return every lane of the group holds the full sum.  SW: source row stride
// in floats (4 for 3-wide vectors, 8 for 8-wide ones).  Every lane of the
// warp must call it (the shuffles are warp-wide).
template <int W, int SW, typename AT>
__device__ __forceinline__ void row_gather(uint32_t lo, uint32_t hi, int sub,
                                           const uint32_t *__restrict__ colidx,
                                           const AT *__restrict__ a,
                                           const float *__restrict__ src, float (&acc)[W]) {
  static_assert(W == 3 || W == 8, "3- or 8-wide gathers");
#pragma unroll
  for (int k = 0; k < W; ++k) acc[k] = 0.f;
  for (uint32_t qb = lo + sub; qb < hi; qb += 16) {
    // entries past the row end reuse the first entry's column with weight 0,
    // so all gathers are unconditional and issue back to back
    float wq[4];
    uint32_t u[4];
    float4 g0[4], g1[4];
    u[0] = __ldg(colidx + qb);
    wq[0] = ldw(a, qb);
#pragma unroll
    for (int k = 1; k < 4; ++k) {
      const uint32_t q = qb + 4 * k;
      const bool ok = q < hi;
      u[k] = ok ? __ldg(colidx + q) : u[0];
      wq[k] = ok ? ldw(a, q) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float4 *s4 = reinterpret_cast<const float4 *>(src + (size_t)u[k] * SW);
      g0[k] = __ldg(s4);
      if (W == 8) g1[k] = __ldg(s4 + 1);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      acc[0] += wq[k] * g0[k].x;
      acc[1] += wq[k] * g0[k].y;
      acc[2] += wq[k] * g0[k].z;
      if (W == 8) {
        acc[3] += wq[k] * g0[k].w;
        acc[4] += wq[k] * g1[k].x;
        acc[5] += wq[k] * g1[k].y;
        acc[6] += wq[k] * g1[k].z;
        acc[7] += wq[k] * g1[k].w;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < W; ++k) {
    acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], 1);
    acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], 2);
  }
}

// Buffers of one folded application.
struct FoldBufs {
  const uint32_t *rowptr, *colidx;
  const void *a;      // FP32 or FP16 edge weights
  const float *g;     // the 7 symmetric 3x3 coefficients G_0..G_6, row-major
  const float *l6;    // packed L^-1 [n][6]
  float *xin;         // x = L^-1 r   [n][4]
  float *w[2];        // Horner partial sums, ping-pong [n][4]
};

constexpr int LG_T = 256;  // threads per CTA of the Horner passes
constexpr int NPOLY = 7;   // polynomial degree 6

// One Horner step w_d = G_d x + Aw w_{d+1} (d = 5 .. 0).  A warp takes 8
// consecutive rows (4 lanes each) per step; the loop condition is
// warp-uniform so every lane reaches the shuffles.  ctl (nullable) gates on
// the solve status (gate) and, after a fallback to block Jacobi, skips the
// polynomial.  LAST (d = 0): z = L^-T w_0 (z = L^-T x = D^-1 r after a
// fallback) and the dot partials of the new z when part != null: r.r at
// part[0 .. np), r.z at part[np .. 2np), z.q at part[2np .. 3np)
// (np = gridDim.x) when want_rr / want_zq, else r.z alone at part[0 .. np).
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
  const int lane = threadIdx.x & 31, sub = lane & 3;
  const int64_t nwarp = (int64_t)gridDim.x * (blockDim.x >> 5);
  DotAcc<float> rr, rz, zq;
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w * 8 < n;
       w += nwarp) {
    const int64_t v = w * 8 + (lane >> 2);
    const bool in = v < n;
    const uint32_t lo = (in && !fb) ? __ldg(B.rowptr + v) : 0u;
    const uint32_t hi = (in && !fb) ? __ldg(B.rowptr + v + 1) : 0u;
    float m[3];
    row_gather<3, 4>(lo, hi, sub, B.colidx, (const AT *)B.a, src, m);
    if (in && sub < 3) {
      const float4 x4 = *reinterpret_cast<const float4 *>(B.xin + v * 4);
      if (!LAST) {
        dst[v * 4 + sub] = (sub == 0 ? m[0] : (sub == 1 ? m[1] : m[2])) + G[sub * 3] * x4.x +
                           G[sub * 3 + 1] * x4.y + G[sub * 3 + 2] * x4.z;
      } else {
        // every lane of the group forms all of w_0 (x after a fallback)
        float w0 = x4.x, w1 = x4.y, w2 = x4.z;
        if (!fb) {
          w0 = m[0] + G[0] * x4.x + G[1] * x4.y + G[2] * x4.z;
          w1 = m[1] + G[3] * x4.x + G[4] * x4.y + G[5] * x4.z;
          w2 = m[2] + G[6] * x4.x + G[7] * x4.y + G[8] * x4.z;
        }
        // (L^-1)^T w, L^-1 = [[l0,0,0],[l1,l2,0],[l3,l4,l5]]
        const float *L = B.l6 + v * 6;
        float zk;
        if (sub == 0) zk = L[0] * w0 + L[1] * w1 + L[3] * w2;
        else if (sub == 1) zk = L[2] * w1 + L[4] * w2;
        else zk = L[5] * w2;
        z[v * 3 + sub] = zk;
        if (part) {
          const float rk = r[v * 3 + sub];
          if (want_rr) rr.add(rk, rk);
          rz.add(rk, zk);
          if (want_zq) zq.add(zk, q[v * 3 + sub]);
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
