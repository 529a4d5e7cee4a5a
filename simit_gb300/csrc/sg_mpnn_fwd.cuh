// Forward passes of the message-passing preconditioner (see sg_mpnn.cuh).
#pragma once
#include "sg_mpnn.cuh"
#include "sg_solver_kernels.cuh"

namespace sg {
namespace mpnn {

// Neighbour gathers run in rounds of GU: each round issues all of its loads
// before the first accumulation, which keeps the sequential sum order.
constexpr int GU = 8;

// ---------------------------------------------------------------------------
// graph data
// ---------------------------------------------------------------------------
template <typename MT>
__global__ void k_diag_norm(int32_t n, const uint32_t *rowptr, const uint32_t *colidx,
                            const MT *vals, float *dn) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = rowptr[v], hi = rowptr[v + 1];
    const uint32_t end = hi;
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (colidx[mid] < (uint32_t)v) lo = mid + 1; else hi = mid;
    }
    float s = 0.f;
    if (lo < end && colidx[lo] == (uint32_t)v)
      for (int k = 0; k < 9; ++k) {
        const float x = (float)vals[(size_t)lo * 9 + k];
        s += x * x;
      }
    dn[v] = sqrtf(s);
  }
}

template <typename MT>
__global__ void k_edge_weights(int32_t n, const uint32_t *rowptr, const uint32_t *colidx,
                               const MT *vals, const float *dn, float *a) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    for (uint32_t q = rowptr[v]; q < rowptr[v + 1]; ++q) {
      const uint32_t c = colidx[q];
      float s = 0.f;
      for (int k = 0; k < 9; ++k) {
        const float x = (float)vals[(size_t)q * 9 + k];
        s += x * x;
      }
      const float den = sqrtf(dn[v] * dn[c]);
      a[q] = (c == (uint32_t)v || !(den > 0.f)) ? 0.f : sqrtf(s) / den;
    }
  }
}

// ---------------------------------------------------------------------------
// F1: s = D^-1 r (and z = s when the solver has fallen back to Jacobi)
// ---------------------------------------------------------------------------
// ctl (may be null): the solver's control block; its fallback flag selects
// Jacobi.  gate != 0: return when the solve is no longer running (inside the
// captured iteration); restarts pass gate = 0.
__global__ void k_f1(const SolveCtl *ctl, int gate, int32_t n, const float *__restrict__ dinv,
                     const float *__restrict__ r, float *__restrict__ s, float *__restrict__ z) {
  if (ctl && gate && ctl->status != ST_RUNNING) return;
  const bool fb = ctl && ctl->fallback;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const float *D = dinv + v * 9;
    const float r0 = r[v * 3], r1 = r[v * 3 + 1], r2 = r[v * 3 + 2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float sk = D[k * 3] * r0 + D[k * 3 + 1] * r1 + D[k * 3 + 2] * r2;
      s[v * 3 + k] = sk;
      if (fb && z) z[v * 3 + k] = sk;
    }
  }
}

// Weights of layer 1 (+P2) staged in shared memory.
struct L1W {
  float w1s[H * 3], w1m[H * 3], p2[K * H];
};

// F2: m1 = sum a s_u; h1 = relu(W1s s + W1m m1); q2 = P2 h1.  One thread per vertex.
__global__ void __launch_bounds__(256) k_f2(const SolveCtl *ctl, int gate, int lin, int32_t n,
                                            const uint32_t *__restrict__ rowptr,
                                            const uint32_t *__restrict__ colidx,
                                            const float *__restrict__ a,
                                            const float *__restrict__ prm,
                                            const float *__restrict__ s, float *__restrict__ m1,
                                            float *__restrict__ q2, float *__restrict__ g1) {
  if (ctl && ((gate && ctl->status != ST_RUNNING) || ctl->fallback)) return;
  __shared__ L1W w;
  for (int i = threadIdx.x; i < H * 3; i += blockDim.x) {
    w.w1s[i] = prm[O_W1S + i];
    w.w1m[i] = prm[O_W1M + i];
  }
  for (int i = threadIdx.x; i < K * H; i += blockDim.x) w.p2[i] = prm[O_P2 + i];
  __syncthreads();
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    float mm0 = 0, mm1 = 0, mm2 = 0;
    const uint32_t qe = rowptr[v + 1];
    for (uint32_t qb = rowptr[v]; qb < qe; qb += GU) {
      float wq[GU], g0[GU], g1[GU], g2[GU];  // all gathers of the round in flight
#pragma unroll
      for (int k = 0; k < GU; ++k)
        if (qb + k < qe) {
          const uint32_t u = colidx[qb + k];
          wq[k] = a[qb + k];
          g0[k] = s[u * 3]; g1[k] = s[u * 3 + 1]; g2[k] = s[u * 3 + 2];
        }
#pragma unroll
      for (int k = 0; k < GU; ++k)
        if (qb + k < qe) {
          mm0 += wq[k] * g0[k];
          mm1 += wq[k] * g1[k];
          mm2 += wq[k] * g2[k];
        }
    }
    const float s0 = s[v * 3], s1 = s[v * 3 + 1], s2 = s[v * 3 + 2];
    m1[v * 3] = mm0;
    m1[v * 3 + 1] = mm1;
    m1[v * 3 + 2] = mm2;
    float qq[K];
#pragma unroll
    for (int j = 0; j < K; ++j) qq[j] = 0.f;
    for (int h = 0; h < H; ++h) {
      const float g = w.w1s[h * 3] * s0 + w.w1s[h * 3 + 1] * s1 + w.w1s[h * 3 + 2] * s2 +
                      w.w1m[h * 3] * mm0 + w.w1m[h * 3 + 1] * mm1 + w.w1m[h * 3 + 2] * mm2;
      if (g1) g1[v * H + h] = g;
      const float hv = (lin & 1) ? g : fmaxf(g, 0.f);
#pragma unroll
      for (int j = 0; j < K; ++j) qq[j] += w.p2[j * H + h] * hv;
    }
#pragma unroll
    for (int j = 0; j < K; ++j) q2[v * K + j] = qq[j];
  }
}

// ---------------------------------------------------------------------------
// F3 / F4: a warp owns 16 consecutive vertices; the 64x64 layers run on the
// tensor cores (mma.sync m16n8k16, bf16 operands, FP32 accumulators).
// lin: bit 0 identity activations; bit 1 split activations (the symmetric
// form): h = bf16(h) + bf16(h - bf16(h)), two products with the same bf16
// weights, so the layer is linear to about 2^-16 and the preconditioner
// stays a fixed symmetric operator to that accuracy.
// ---------------------------------------------------------------------------
constexpr int TC_WARPS = 4;
constexpr int HP = H + 8;  // padded bf16 row (36 words: conflict-free fragments)

__device__ __forceinline__ void mma_bf16(float *d, uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// acc[nt][4] += X (16 x 64, bf16, row stride HP) * W^T (W: 64 x 64 bf16, row stride HP)
__device__ __forceinline__ void gemm16x64(const __nv_bfloat16 *X, const __nv_bfloat16 *W,
                                          float acc[8][4]) {
  const int lane = threadIdx.x & 31, gid = lane >> 2, t = lane & 3;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    const int k0 = kk * 16;
    const uint32_t a0 = *reinterpret_cast<const uint32_t *>(X + gid * HP + k0 + 2 * t);
    const uint32_t a1 = *reinterpret_cast<const uint32_t *>(X + (gid + 8) * HP + k0 + 2 * t);
    const uint32_t a2 = *reinterpret_cast<const uint32_t *>(X + gid * HP + k0 + 2 * t + 8);
    const uint32_t a3 = *reinterpret_cast<const uint32_t *>(X + (gid + 8) * HP + k0 + 2 * t + 8);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const __nv_bfloat16 *wr = W + (nt * 8 + gid) * HP + k0 + 2 * t;
      const uint32_t b0 = *reinterpret_cast<const uint32_t *>(wr);
      const uint32_t b1 = *reinterpret_cast<const uint32_t *>(wr + 8);
      mma_bf16(acc[nt], a0, a1, a2, a3, b0, b1);
    }
  }
}

struct TCW {
  __nv_bfloat16 w2h[H * HP];
  __nv_bfloat16 w3h[H * HP];
  float w1s[H * 3], w1m[H * 3], w2m[H * K], w3m[H * K], p3[K * H], wout[3 * H];
  float wx[3 * H];  // extra output projection (F4 of the transposed network)
};
struct TCWarp {
  __nv_bfloat16 x1[16 * HP];
  __nv_bfloat16 x2[16 * HP];
  __nv_bfloat16 x1lo[16 * HP];  // split activations: bf16(h - bf16(h))
  __nv_bfloat16 x2lo[16 * HP];
  float mA[16 * K];  // m2 (F3) or m3 (F4)
  float mB[16 * K];  // m2 (F4)
  float sv[16 * 3], m1v[16 * 3];
};

__device__ __forceinline__ void load_tc_weights(TCW &w, const float *prm, bool need_w3) {
  for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
    const int r = i / H, c = i % H;
    w.w2h[r * HP + c] = __float2bfloat16_rn(prm[O_W2H + i]);
    if (need_w3) w.w3h[r * HP + c] = __float2bfloat16_rn(prm[O_W3H + i]);
  }
  for (int i = threadIdx.x; i < H * 3; i += blockDim.x) {
    w.w1s[i] = prm[O_W1S + i];
    w.w1m[i] = prm[O_W1M + i];
    w.wout[i] = prm[O_WOUT + i];
  }
  for (int i = threadIdx.x; i < H * K; i += blockDim.x) {
    w.w2m[i] = prm[O_W2M + i];
    w.w3m[i] = prm[O_W3M + i];
    w.p3[i] = prm[O_P3 + i];
  }
}

// The warp's 16 vertices: gather m = sum a q_u (8-dim) into dst[16*K]; load
// s and m1; rebuild bf16(h1) into x1.
__device__ __forceinline__ void tc_prologue(const TCW &w, TCWarp &tw, int lin, int64_t v0, int32_t n,
                                            const uint32_t *rowptr, const uint32_t *colidx,
                                            const float *a, const float *qsrc, float *dst,
                                            const float *s, const float *m1) {
  const int lane = threadIdx.x & 31;
  {
    const int vi = lane & 15, half = lane >> 4;
    const int64_t v = v0 + vi;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (v < n) {
      const uint32_t qe = rowptr[v + 1];
      for (uint32_t qb = rowptr[v]; qb < qe; qb += GU) {
        float wq[GU];
        float4 xg[GU];  // all gathers of the round in flight
#pragma unroll
        for (int k = 0; k < GU; ++k)
          if (qb + k < qe) {
            wq[k] = a[qb + k];
            xg[k] = *reinterpret_cast<const float4 *>(qsrc + (size_t)colidx[qb + k] * K + half * 4);
          }
#pragma unroll
        for (int k = 0; k < GU; ++k)
          if (qb + k < qe) {
            acc.x += wq[k] * xg[k].x;
            acc.y += wq[k] * xg[k].y;
            acc.z += wq[k] * xg[k].z;
            acc.w += wq[k] * xg[k].w;
          }
      }
    }
    dst[vi * K + half * 4 + 0] = acc.x;
    dst[vi * K + half * 4 + 1] = acc.y;
    dst[vi * K + half * 4 + 2] = acc.z;
    dst[vi * K + half * 4 + 3] = acc.w;
  }
  for (int i = lane; i < 16 * 3; i += 32) {
    const int64_t v = v0 + i / 3;
    tw.sv[i] = v < n ? s[v0 * 3 + i] : 0.f;
    tw.m1v[i] = v < n ? m1[v0 * 3 + i] : 0.f;
  }
  __syncwarp();
  {
    const int vi = lane & 15, h0 = (lane >> 4) * 32;
    const float *sv = tw.sv + vi * 3, *mv = tw.m1v + vi * 3;
    for (int h = h0; h < h0 + 32; ++h) {
      const float g = w.w1s[h * 3] * sv[0] + w.w1s[h * 3 + 1] * sv[1] + w.w1s[h * 3 + 2] * sv[2] +
                      w.w1m[h * 3] * mv[0] + w.w1m[h * 3 + 1] * mv[1] + w.w1m[h * 3 + 2] * mv[2];
      const float hv = (lin & 1) ? g : fmaxf(g, 0.f);
      const __nv_bfloat16 hi = __float2bfloat16_rn(hv);
      tw.x1[vi * HP + h] = hi;
      if (lin & 2) tw.x1lo[vi * HP + h] = __float2bfloat16_rn(hv - __bfloat162float(hi));
    }
  }
  __syncwarp();
}

// Epilogue of a 64x64 layer: acc += Wm m (m from msrc[16*K]); optional store
// of the pre-activation g; acc <- relu(acc).
__device__ __forceinline__ void tc_layer_epilogue(float acc[8][4], const float *Wm,
                                                  const float *msrc, int64_t v0, int32_t n,
                                                  float *g_out, int lin) {
  const int lane = threadIdx.x & 31, gid = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int row = gid + (e >> 1) * 8, col = nt * 8 + 2 * t + (e & 1);
      float gsum = acc[nt][e];
#pragma unroll
      for (int j = 0; j < K; ++j) gsum += Wm[col * K + j] * msrc[row * K + j];
      if (g_out && v0 + row < n) g_out[(v0 + row) * H + col] = gsum;
      acc[nt][e] = (lin & 1) ? gsum : fmaxf(gsum, 0.f);
    }
}

// F3: m2 = sum a q2_u; g2 = W2h bf16(h1) + W2m m2; h2 = relu(g2); q3 = P3 h2.
__global__ void __launch_bounds__(TC_WARPS * 32)
    k_f3(const SolveCtl *ctl, int gate, int lin, int32_t n, const uint32_t *__restrict__ rowptr,
         const uint32_t *__restrict__ colidx, const float *__restrict__ a,
         const float *__restrict__ prm, const float *__restrict__ s,
         const float *__restrict__ m1, const float *__restrict__ q2, float *__restrict__ m2,
         float *__restrict__ q3, float *__restrict__ g2) {
  if (ctl && ((gate && ctl->status != ST_RUNNING) || ctl->fallback)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  TCW &w = *reinterpret_cast<TCW *>(smraw);
  TCWarp &tw = reinterpret_cast<TCWarp *>(smraw + sizeof(TCW))[threadIdx.x >> 5];
  load_tc_weights(w, prm, false);
  __syncthreads();
  const int lane = threadIdx.x & 31, gid = lane >> 2, t = lane & 3;
  const int64_t ntile = ((int64_t)n + 15) / 16;
  for (int64_t tile = (int64_t)blockIdx.x * TC_WARPS + (threadIdx.x >> 5); tile < ntile;
       tile += (int64_t)gridDim.x * TC_WARPS) {
    const int64_t v0 = tile * 16;
    tc_prologue(w, tw, lin, v0, n, rowptr, colidx, a, q2, tw.mA, s, m1);
    for (int i = lane; i < 16 * K; i += 32)
      if (v0 + i / K < n) m2[v0 * K + i] = tw.mA[i];
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[nt][e] = 0.f;
    gemm16x64(tw.x1, w.w2h, acc);
    if (lin & 2) gemm16x64(tw.x1lo, w.w2h, acc);
    tc_layer_epilogue(acc, w.w2m, tw.mA, v0, n, g2, lin);
    // q3[row][j] = sum_n P3[j][n] h2[row][n]: quad partials then shuffles
    float qa[K], qb[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      float pa = 0.f, pb = 0.f;
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int col = nt * 8 + 2 * t + e;
          pa += w.p3[j * H + col] * acc[nt][e];
          pb += w.p3[j * H + col] * acc[nt][2 + e];
        }
      pa += __shfl_xor_sync(0xffffffffu, pa, 1);
      pa += __shfl_xor_sync(0xffffffffu, pa, 2);
      pb += __shfl_xor_sync(0xffffffffu, pb, 1);
      pb += __shfl_xor_sync(0xffffffffu, pb, 2);
      qa[j] = pa;
      qb[j] = pb;
    }
    if (t == 0) {
      if (v0 + gid < n)
#pragma unroll
        for (int j = 0; j < K; ++j) q3[(v0 + gid) * K + j] = qa[j];
      if (v0 + gid + 8 < n)
#pragma unroll
        for (int j = 0; j < K; ++j) q3[(v0 + gid + 8) * K + j] = qb[j];
    }
    __syncwarp();
  }
}

// F4: m3 = sum a q3_u; h2 = relu(W2h bf16(h1) + W2m m2); g3 = W3h bf16(h2) +
// W3m m3; h3 = relu(g3); z = s + Wout h3.  With wx_prm (the untransposed
// parameters, for the transposed network) also tout = W1m^T h3.
__global__ void __launch_bounds__(TC_WARPS * 32)
    k_f4(const SolveCtl *ctl, int gate, int lin, int32_t n, const uint32_t *__restrict__ rowptr,
         const uint32_t *__restrict__ colidx, const float *__restrict__ a,
         const float *__restrict__ prm, const float *__restrict__ s,
         const float *__restrict__ m1, const float *__restrict__ m2,
         const float *__restrict__ q3, float *__restrict__ m3, float *__restrict__ z,
         float *__restrict__ g3, const float *__restrict__ wx_prm = nullptr,
         float *__restrict__ tout = nullptr) {
  if (ctl && ((gate && ctl->status != ST_RUNNING) || ctl->fallback)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  TCW &w = *reinterpret_cast<TCW *>(smraw);
  TCWarp &tw = reinterpret_cast<TCWarp *>(smraw + sizeof(TCW))[threadIdx.x >> 5];
  load_tc_weights(w, prm, true);
  if (wx_prm)
    for (int i = threadIdx.x; i < 3 * H; i += blockDim.x) {
      const int k = i / H, h = i % H;
      w.wx[i] = wx_prm[O_W1M + h * 3 + k];
    }
  __syncthreads();
  const int lane = threadIdx.x & 31, gid = lane >> 2, t = lane & 3;
  const int64_t ntile = ((int64_t)n + 15) / 16;
  for (int64_t tile = (int64_t)blockIdx.x * TC_WARPS + (threadIdx.x >> 5); tile < ntile;
       tile += (int64_t)gridDim.x * TC_WARPS) {
    const int64_t v0 = tile * 16;
    tc_prologue(w, tw, lin, v0, n, rowptr, colidx, a, q3, tw.mA, s, m1);
    for (int i = lane; i < 16 * K; i += 32) {
      const bool in = v0 + i / K < n;
      tw.mB[i] = in ? m2[v0 * K + i] : 0.f;
      if (in) m3[v0 * K + i] = tw.mA[i];
    }
    __syncwarp();
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[nt][e] = 0.f;
    gemm16x64(tw.x1, w.w2h, acc);
    if (lin & 2) gemm16x64(tw.x1lo, w.w2h, acc);
    tc_layer_epilogue(acc, w.w2m, tw.mB, v0, n, nullptr, lin);
    // h2 -> bf16 tile x2
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int row = gid + (e >> 1) * 8, col = nt * 8 + 2 * t + (e & 1);
        const __nv_bfloat16 hi = __float2bfloat16_rn(acc[nt][e]);
        tw.x2[row * HP + col] = hi;
        if (lin & 2) tw.x2lo[row * HP + col] = __float2bfloat16_rn(acc[nt][e] - __bfloat162float(hi));
      }
    __syncwarp();
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[nt][e] = 0.f;
    gemm16x64(tw.x2, w.w3h, acc);
    if (lin & 2) gemm16x64(tw.x2lo, w.w3h, acc);
    tc_layer_epilogue(acc, w.w3m, tw.mA, v0, n, g3, lin);
    float za[3], zb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float pa = 0.f, pb = 0.f;
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int col = nt * 8 + 2 * t + e;
          pa += w.wout[k * H + col] * acc[nt][e];
          pb += w.wout[k * H + col] * acc[nt][2 + e];
        }
      pa += __shfl_xor_sync(0xffffffffu, pa, 1);
      pa += __shfl_xor_sync(0xffffffffu, pa, 2);
      pb += __shfl_xor_sync(0xffffffffu, pb, 1);
      pb += __shfl_xor_sync(0xffffffffu, pb, 2);
      za[k] = pa;
      zb[k] = pb;
    }
    if (t == 0) {
      if (v0 + gid < n)
#pragma unroll
        for (int k = 0; k < 3; ++k) z[(v0 + gid) * 3 + k] = tw.sv[gid * 3 + k] + za[k];
      if (v0 + gid + 8 < n)
#pragma unroll
        for (int k = 0; k < 3; ++k) z[(v0 + gid + 8) * 3 + k] = tw.sv[(gid + 8) * 3 + k] + zb[k];
    }
    if (wx_prm) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float pa = 0.f, pb = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int col = nt * 8 + 2 * t + e;
            pa += w.wx[k * H + col] * acc[nt][e];
            pb += w.wx[k * H + col] * acc[nt][2 + e];
          }
        pa += __shfl_xor_sync(0xffffffffu, pa, 1);
        pa += __shfl_xor_sync(0xffffffffu, pa, 2);
        pb += __shfl_xor_sync(0xffffffffu, pb, 1);
        pb += __shfl_xor_sync(0xffffffffu, pb, 2);
        za[k] = pa;
        zb[k] = pb;
      }
      if (t == 0) {
        if (v0 + gid < n)
#pragma unroll
          for (int k = 0; k < 3; ++k) tout[(v0 + gid) * 3 + k] = za[k];
        if (v0 + gid + 8 < n)
#pragma unroll
          for (int k = 0; k < 3; ++k) tout[(v0 + gid + 8) * 3 + k] = zb[k];
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Symmetric factorized form
// ---------------------------------------------------------------------------
// L_v^-1 (row-major 3x3, lower triangular) with D_v = L_v L_v^T, in FP64
// from the lower triangle of the diagonal block.  A block that is not
// positive definite gets diag(1/sqrt|d_kk|) (0 for d_kk = 0).
template <typename MT>
__global__ void k_chol_inv(int32_t n, const uint32_t *rowptr, const uint32_t *colidx,
                           const MT *vals, float *linv) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = rowptr[v], hi = rowptr[v + 1];
    const uint32_t end = hi;
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (colidx[mid] < (uint32_t)v) lo = mid + 1; else hi = mid;
    }
    double d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (lo < end && colidx[lo] == (uint32_t)v)
      for (int k = 0; k < 9; ++k) d[k] = (double)vals[(size_t)lo * 9 + k];
    double x[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double l00 = sqrt(d[0]);
    const double l10 = d[3] / l00, l20 = d[6] / l00;
    const double t11 = d[4] - l10 * l10;
    const double l11 = sqrt(t11);
    const double l21 = (d[7] - l20 * l10) / l11;
    const double t22 = d[8] - l20 * l20 - l21 * l21;
    const double l22 = sqrt(t22);
    if (d[0] > 0 && t11 > 0 && t22 > 0 && isfinite(l22)) {
      // solve L X = I column by column
      x[0] = 1.0 / l00;
      x[3] = -l10 * x[0] / l11;
      x[6] = -(l20 * x[0] + l21 * x[3]) / l22;
      x[4] = 1.0 / l11;
      x[7] = -l21 * x[4] / l22;
      x[8] = 1.0 / l22;
    } else {
      for (int k = 0; k < 3; ++k) {
        const double a = fabs(d[k * 4]);
        x[k * 4] = a > 0 ? 1.0 / sqrt(a) : 0.0;
      }
    }
    for (int k = 0; k < 9; ++k) linv[(size_t)v * 9 + k] = (float)x[k];
  }
}

// Parameters of the transposed network (same flat layout): layer 1 <- Wout^T
// with no message, layer 2 <- layer 3 transposed, layer 3 <- layer 2
// transposed, output <- W1s^T.
__global__ void k_transpose_params(const float *__restrict__ p, float *__restrict__ q) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NPARAM; i += gridDim.x * blockDim.x) {
    float v;
    if (i < O_W1M) { const int h = (i - O_W1S) / 3, k = (i - O_W1S) % 3; v = p[O_WOUT + k * H + h]; }
    else if (i < O_P2) v = 0.f;
    else if (i < O_W2H) { const int j = (i - O_P2) / H, h = (i - O_P2) % H; v = p[O_W3M + h * K + j]; }
    else if (i < O_W2M) { const int r = (i - O_W2H) / H, c = (i - O_W2H) % H; v = p[O_W3H + c * H + r]; }
    else if (i < O_P3) { const int h = (i - O_W2M) / K, j = (i - O_W2M) % K; v = p[O_P3 + j * H + h]; }
    else if (i < O_W3H) { const int j = (i - O_P3) / H, h = (i - O_P3) % H; v = p[O_W2M + h * K + j]; }
    else if (i < O_W3M) { const int r = (i - O_W3H) / H, c = (i - O_W3H) % H; v = p[O_W2H + c * H + r]; }
    else if (i < O_WOUT) { const int h = (i - O_W3M) / K, j = (i - O_W3M) % K; v = p[O_P2 + j * H + h]; }
    else { const int k = (i - O_WOUT) / H, h = (i - O_WOUT) % H; v = p[O_W1S + h * 3 + k]; }
    q[i] = v;
  }
}

// z_v = L_v^-T (wp_v + sum_u a_vu t_u); after a fallback z_v = L_v^-T s_v
// (= D_v^-1 r_v, block Jacobi).
__global__ void k_sym_out(const SolveCtl *ctl, int gate, int32_t n,
                          const uint32_t *__restrict__ rowptr, const uint32_t *__restrict__ colidx,
                          const float *__restrict__ a, const float *__restrict__ linv,
                          const float *__restrict__ wp, const float *__restrict__ t,
                          const float *__restrict__ s, float *__restrict__ z) {
  if (ctl && gate && ctl->status != ST_RUNNING) return;
  const bool fb = ctl && ctl->fallback;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    float w0, w1, w2;
    if (fb) {
      w0 = s[v * 3]; w1 = s[v * 3 + 1]; w2 = s[v * 3 + 2];
    } else {
      w0 = wp[v * 3]; w1 = wp[v * 3 + 1]; w2 = wp[v * 3 + 2];
      const uint32_t qe = rowptr[v + 1];
      for (uint32_t qb = rowptr[v]; qb < qe; qb += GU) {
        float aq[GU], g0[GU], g1[GU], g2[GU];
#pragma unroll
        for (int k = 0; k < GU; ++k)
          if (qb + k < qe) {
            const uint32_t u = colidx[qb + k];
            aq[k] = a[qb + k];
            g0[k] = t[(size_t)u * 3]; g1[k] = t[(size_t)u * 3 + 1]; g2[k] = t[(size_t)u * 3 + 2];
          }
#pragma unroll
        for (int k = 0; k < GU; ++k)
          if (qb + k < qe) {
            w0 += aq[k] * g0[k];
            w1 += aq[k] * g1[k];
            w2 += aq[k] * g2[k];
          }
      }
    }
    const float *Li = linv + (size_t)v * 9;
#pragma unroll
    for (int k = 0; k < 3; ++k) z[v * 3 + k] = Li[k] * w0 + Li[3 + k] * w1 + Li[6 + k] * w2;
  }
}

__global__ void k_add_f(int n, float *__restrict__ a, const float *__restrict__ b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    a[i] += b[i];
}

inline size_t tc_smem_bytes() { return sizeof(TCW) + TC_WARPS * sizeof(TCWarp); }

}  // namespace mpnn
}  // namespace sg
