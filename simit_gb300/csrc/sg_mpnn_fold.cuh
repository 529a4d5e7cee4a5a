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
// x = L^-1 r (fused into the iteration's r update), six Horner steps
// w_d = G_d x + Aw w_{d+1} (w_6 = G_6 x, applied after the first step's
// gather), each a gather of a 3-wide vector over the matrix pattern, and
// z = L^-T w_0 with the iteration's dot products fused into the last step -- instead of twelve 64x64 tensor-core
// products per 16-vertex tile and seven gather passes of up to 8-wide
// messages.  The operator is the one the layered kernels evaluate (their
// split-bf16 activations carry the hidden layers to about 2^-16); tests
// compare the two and the oracle's restatement.
//
// Layout: x and the Horner sums are [n][4] (float4 per vertex); the passes
// read the pattern and the edge weights (FP16 by default, FP32 on request)
// from a sliced-ELLPACK copy with one lane per row (SellGraph below).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "sg_mpnn.cuh"
#include "sg_solver_kernels.cuh"
#include "sg_tma.cuh"

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
// 9-value form k_chol_inv writes: FP32 for the FP32 evaluation (l6) and
// BF16, rounded to nearest even, for the FP16 one (l6b, 12 bytes per vertex:
// the factor is read twice per application, by x = L^-1 r and z = L^-T w_0,
// and both read the same rounded factor, so M stays exactly symmetric).
__global__ void k_pack_linv(int32_t n, const float *__restrict__ linv, float *__restrict__ l6,
                            uint32_t *__restrict__ l6b) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const float *L = linv + v * 9;
    const float o[6] = {L[0], L[3], L[4], L[6], L[7], L[8]};
    for (int k = 0; k < 6; ++k) l6[v * 6 + k] = o[k];
    for (int k = 0; k < 3; ++k)
      l6b[v * 3 + k] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(o[2 * k])) |
                       ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(o[2 * k + 1])) << 16);
  }
}

// L_v^-1 of one vertex (6 packed values) from the evaluation's copy: BF16
// pairs (low half first) when CV, else FP32.
template <bool CV>
__device__ __forceinline__ void ld_linv(const void *__restrict__ l6, size_t v, float *L) {
  if (CV) {
    const uint32_t *p = reinterpret_cast<const uint32_t *>(l6) + v * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint32_t u = __ldg(p + k);
      L[2 * k] = __uint_as_float(u << 16);
      L[2 * k + 1] = __uint_as_float(u & 0xffff0000u);
    }
  } else {
    const float *p = reinterpret_cast<const float *>(l6) + v * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) L[k] = p[k];
  }
}
// The same for vertices 4u .. 4u+3 (24 values) with 16-byte loads: three
// when CV (48 bytes), else six.
template <bool CV>
__device__ __forceinline__ void ld_linv4(const void *__restrict__ l6, int64_t u, float *lv) {
  if (CV) {
    const uint4 *p = reinterpret_cast<const uint4 *>(l6) + u * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint4 g = __ldg(p + k);
      const uint32_t w[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        lv[8 * k + 2 * j] = __uint_as_float(w[j] << 16);
        lv[8 * k + 2 * j + 1] = __uint_as_float(w[j] & 0xffff0000u);
      }
    }
  } else {
    const float4 *p = reinterpret_cast<const float4 *>(l6) + u * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float4 g = p[k];
      lv[4 * k] = g.x; lv[4 * k + 1] = g.y; lv[4 * k + 2] = g.z; lv[4 * k + 3] = g.w;
    }
  }
}

__device__ __forceinline__ float tofloat(float w) { return w; }
__device__ __forceinline__ float tofloat(__half w) { return __half2float(w); }

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
constexpr uint32_t SL_NONE = 0xffffffffu;
constexpr int LG_T = 256;         // threads per CTA of the finish kernel
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

// Blocks of the finish kernel of an application over `nslice` slices of
// rows (also the number of dot partials it leaves in the solver).
inline int finish_grid(const Ctx *c, int32_t nslice) {
  return grid_for(c, (int64_t)nslice * SL_W, LG_T, 8);
}

// Vectors of the FP16 evaluation.  x and the Horner sums are stored per
// vertex as three FP16 mantissas with a shared power-of-two exponent (block
// floating point, 8 bytes): value = h * 2^e, the largest |h| in [0.5, 1).
// A gather then reads 8 bytes per neighbour instead of 16, each vertex keeps
// 11 significant bits relative to its largest component, and the shared
// exponent (a 16-bit integer) covers any FP32 magnitude -- residuals
// shrink by many orders during a solve, which plain FP16 would underflow.
// Values below 2^-24 of their vertex's largest are stored as 0; a
// non-finite value is stored as such and propagates.  The FP32 evaluation
// keeps float4 vectors.
__device__ __forceinline__ float pow2f(int e) {  // 2^e, e in [-126, 127]
  return __int_as_float((127 + e) << 23);
}
__device__ __forceinline__ uint2 cv_encode(float a, float b, float c) {
  const float m = fmaxf(fabsf(a), fmaxf(fabsf(b), fabsf(c)));
  const int mb = __float_as_int(m);
  int e = 0;
  float s = 1.f;
  // normal, finite m: m = f 2^e with f in [0.5, 1); keep 2^-e representable
  if (mb >= 0x00800000 && mb < 0x7f800000) {
    e = ((mb >> 23) & 0xff) - 126;
    e = e < -125 ? -125 : (e > 126 ? 126 : e);
    s = pow2f(-e);
  } else if (mb < 0x00800000) {
    a = b = c = 0.f;  // zero or FP32-subnormal: stored as 0
  }
  uint2 u;
  u.x = (uint32_t)__half_as_ushort(__float2half_rn(a * s)) |
        ((uint32_t)__half_as_ushort(__float2half_rn(b * s)) << 16);
  u.y = (uint32_t)__half_as_ushort(__float2half_rn(c * s)) | ((uint32_t)(uint16_t)(int16_t)e << 16);
  return u;
}
__device__ __forceinline__ void cv_decode(uint2 u, float &a, float &b, float &c) {
  const float s = pow2f((int)(int16_t)(u.y >> 16));
  a = __half2float(__ushort_as_half((unsigned short)(u.x & 0xffffu))) * s;
  b = __half2float(__ushort_as_half((unsigned short)(u.x >> 16))) * s;
  c = __half2float(__ushort_as_half((unsigned short)(u.y & 0xffffu))) * s;
}

// A vertex's three values from / to a vector of the evaluation (CV: block
// floating point, else float4).
template <bool CV>
__device__ __forceinline__ void ld3(const void *__restrict__ p, size_t v, float &a, float &b,
                                    float &c) {
  if (CV) {
    cv_decode(__ldg(reinterpret_cast<const uint2 *>(p) + v), a, b, c);
  } else {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(p) + v);
    a = t.x;
    b = t.y;
    c = t.z;
  }
}
template <bool CV>
__device__ __forceinline__ void st3(void *__restrict__ p, size_t v, float a, float b, float c) {
  if (CV) reinterpret_cast<uint2 *>(p)[v] = cv_encode(a, b, c);
  else reinterpret_cast<float4 *>(p)[v] = make_float4(a, b, c, 0.f);
}

// Buffers of one folded application.  x and the Horner sums hold 16 bytes
// per vertex: float4 in the FP32 evaluation, the first 8 in block floating
// point in the FP16 one.
struct FoldBufs {
  SellGraph sl;
  const void *a;      // FP32 or FP16 edge weights in slice order
  const float *g;     // the 7 symmetric 3x3 coefficients G_0..G_6, row-major
  const float *l6;    // packed L^-1 [n][6], FP32 (the FP32 evaluation)
  const uint32_t *l6b;  // the same in BF16 [n][6] (the FP16 evaluation)
  void *xin;          // x = L^-1 r
  void *w[2];         // Horner partial sums, ping-pong
};

// One Horner step w_d = G_d x + Aw w_{d+1} (d = 5 .. 0).  The first step
// (first != 0, d = 5) gathers x itself and applies G_6 to the sum:
// Aw (G_6 x) = G_6 (Aw x) at every vertex, so w_6 is never stored.  A warp
// takes one slice (a lane per row) at a time.  The slice's indices and
// weights are staged in shared memory by bulk copies (cp.async.bulk +
// mbarrier), HT_NST slices in flight per warp, so the gathers of one slice
// overlap the copies of the next.  A slice's indices and weights are
// contiguous and 128- / 64-byte aligned (slices start at multiples of 32
// entries), so each is one copy with no tail; slices longer than HT_CAPL
// entries per lane are read from global memory.  Every barrier wait is
// bounded: on a timeout the warp records DEV_TMA_TIMEOUT in err, waits
// (bounded) for its copies in flight and stops.  ctl (nullable) gates on
// the solve status (gate); after a fallback to block Jacobi the steps do
// nothing (k_lrn_finish then uses x).  AT: edge-weight type; FP16 weights
// go with block-floating-point vectors.
// The end of an application folded into the last Horner step (FIN): each
// row's w_0 becomes z = L^-T w_0 at once, and the dots r.r, r.z, z.q of the
// new z accumulate as it goes, one partial per CTA (grid-size apart, as
// k_lrn_finish leaves them).  part null: z alone.
struct FinArgs {
  const float *r = nullptr;
  const float *q = nullptr;
  float *z = nullptr;
  double *part = nullptr;
  int want_rr = 0, want_zq = 0;
  // decide (with all three dots): the CTA that finishes last also sums the
  // partials and makes the iteration's decision (cg_decide: status, beta)
  // for K3, which then only streams
  SolveCtl *ctl = nullptr;
  int decide = 0, par = 0;
};

constexpr int HT_WARPS = 4;   // warps per CTA
constexpr int HT_NST = 2;     // slices in flight per warp
constexpr int HT_CAPL = 20;   // longest staged slice (entries per lane)

template <typename AT>
__host__ __device__ constexpr size_t ht_stage_bytes() {
  return (size_t)HT_CAPL * SL_W * (4 + sizeof(AT));
}
template <typename AT>
__host__ __device__ constexpr size_t ht_smem_bytes() {
  return (((size_t)HT_WARPS * HT_NST * 8 + 15) & ~size_t(15)) +
         (size_t)HT_WARPS * HT_NST * ht_stage_bytes<AT>();
}

template <typename AT, bool FIN = false>
__global__ void __launch_bounds__(HT_WARPS * 32, FIN ? 7 : 1)
    k_horner(const SolveCtl *ctl, int gate, FoldBufs B, int d,
                 const void *__restrict__ src, void *__restrict__ dst, int first, int *err,
                 FinArgs fa = FinArgs()) {
  constexpr bool CV = sizeof(AT) == 2;
  constexpr size_t CB = (size_t)HT_CAPL * SL_W * 4;
  constexpr size_t STG = ht_stage_bytes<AT>();
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ float G[9], G6[9];
  __shared__ double shd[33];
  if (ctl && gate && ctl->status != ST_RUNNING) return;
  // after a fallback to block Jacobi the steps do nothing, and the last one
  // (FIN) turns x itself into z = L^-T x
  const bool fb = ctl && ctl->fallback;
  if (fb && !FIN) return;
  DotAcc<float> rr, rz, zq;
  auto fin = [&](uint32_t v, float a, float b, float c) {
    // z = (L^-1)^T w, L^-1 = [[l0,0,0],[l1,l2,0],[l3,l4,l5]], as k_lrn_finish
    float L[6];
    ld_linv<CV>(CV ? (const void *)B.l6b : (const void *)B.l6, v, L);
    const float z0 = L[0] * a + L[1] * b + L[3] * c;
    const float z1 = L[2] * b + L[4] * c;
    const float z2 = L[5] * c;
    float *zp = fa.z + (size_t)v * 3;
    zp[0] = z0;
    zp[1] = z1;
    zp[2] = z2;
    if (!fa.part) return;
    const float *rp = fa.r + (size_t)v * 3;
    const float r0 = rp[0], r1 = rp[1], r2 = rp[2];
    if (fa.want_rr) {
      rr.add(r0, r0);
      rr.add(r1, r1);
      rr.add(r2, r2);
    }
    rz.add(r0, z0);
    rz.add(r1, z1);
    rz.add(r2, z2);
    if (fa.want_zq) {
      const float *qp = fa.q + (size_t)v * 3;
      zq.add(z0, qp[0]);
      zq.add(z1, qp[1]);
      zq.add(z2, qp[2]);
    }
  };
  auto fin_partials = [&]() {
    if (!FIN || !fa.part) return;
    const double t1 = block_sum(rz.value(), shd);
    const double t0 = fa.want_rr ? block_sum(rr.value(), shd) : 0.0;
    const double t2 = fa.want_zq ? block_sum(zq.value(), shd) : 0.0;
    if (fa.decide) {
      // r.r | r.z | z.q, each gridDim.x partials, summed in index order by
      // the last CTA, which decides the iteration
      const double t[3] = {t0, t1, t2};
      double tot[3];
      if (finalize_partials(t, 3, fa.part, &fa.ctl->tick2, tot, shd) && threadIdx.x == 0)
        cg_decide(fa.ctl, fa.par, tot[0], tot[1], tot[2], fa.ctl->last_alpha);
      return;
    }
    if (threadIdx.x == 0) {
      if (fa.want_rr) fa.part[blockIdx.x] = t0;
      fa.part[(fa.want_rr ? gridDim.x : 0) + blockIdx.x] = t1;
      if (fa.want_zq) fa.part[2 * gridDim.x + blockIdx.x] = t2;
    }
  };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (FIN && fb) {
    // the slices as the steps take them, each row's x straight to z
    const int64_t ns = B.sl.nslice;
    for (int64_t s = (int64_t)blockIdx.x * HT_WARPS + warp; s < ns;
         s += (int64_t)gridDim.x * HT_WARPS) {
      const uint32_t v = __ldg(B.sl.row + s * SL_W + lane);
      if (v == SL_NONE) continue;
      float x0, x1, x2;
      ld3<CV>(B.xin, v, x0, x1, x2);
      fin(v, x0, x1, x2);
    }
    fin_partials();
    return;
  }
  if (threadIdx.x < 9) G[threadIdx.x] = B.g[d * 9 + threadIdx.x];
  else if (threadIdx.x < 18) G6[threadIdx.x - 9] = B.g[6 * 9 + threadIdx.x - 9];
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm) + warp * HT_NST;
  unsigned char *base =
      sm + (((size_t)HT_WARPS * HT_NST * 8 + 15) & ~size_t(15)) + (size_t)warp * HT_NST * STG;
  if (lane == 0) {
    for (int b = 0; b < HT_NST; ++b) mbar_init(&bar[b], 1);
    mbar_fence_init();
  }
  __syncthreads();
  const AT *__restrict__ aw = (const AT *)B.a;
  const int64_t ns = B.sl.nslice;
  const int64_t gw = (int64_t)blockIdx.x * HT_WARPS + warp;
  const int64_t nw = (int64_t)gridDim.x * HT_WARPS;
  const int64_t my = gw < ns ? (ns - 1 - gw) / nw + 1 : 0;
  // lane 0: stage slice s in buffer b (or arrive with no bytes when it is
  // empty or longer than the buffer)
  auto issue = [&](int64_t s, int b) {
    const uint32_t p0 = B.sl.ptr[s], p1 = B.sl.ptr[s + 1];
    const uint32_t len = (p1 - p0) / SL_W;
    fence_proxy_async_smem();
    if (len == 0 || len > (uint32_t)HT_CAPL) {
      mbar_arrive_expect_tx(&bar[b], 0);
      return;
    }
    const uint32_t cb = len * SL_W * 4, wb = len * SL_W * (uint32_t)sizeof(AT);
    mbar_arrive_expect_tx(&bar[b], cb + wb);
    bulk_g2s(base + (size_t)b * STG, B.sl.col + p0, cb, &bar[b]);
    bulk_g2s(base + (size_t)b * STG + CB, aw + p0, wb, &bar[b]);
  };
  if (lane == 0)
    for (int k = 0; k < HT_NST - 1 && k < my; ++k) issue(gw + k * nw, k);
  for (int64_t k = 0; k < my; ++k) {
    const int b = (int)(k % HT_NST);
    const int64_t s = gw + k * nw;
    const int64_t kn = k + HT_NST - 1;
    if (lane == 0 && kn < my) issue(gw + kn * nw, (int)(kn % HT_NST));
    const bool ok = __all_sync(0xffffffffu, mbar_wait(&bar[b], (uint32_t)((k / HT_NST) & 1)));
    if (!ok) {
      if (lane == 0) {
        atomicCAS(err, 0, 6 /* DEV_TMA_TIMEOUT */);
        bool drained = true;
        for (int64_t kk = k; kk < my && kk <= kn; ++kk)
          drained = mbar_wait(&bar[kk % HT_NST], (uint32_t)((kk / HT_NST) & 1)) && drained;
        if (!drained) atomicExch(err, 8 /* DEV_TMA_UNDRAINED */);
      }
      break;
    }
    const uint32_t v = __ldg(B.sl.row + s * SL_W + lane);
    const uint32_t p0 = __ldg(B.sl.ptr + s), p1 = __ldg(B.sl.ptr + s + 1);
    const uint32_t len = (p1 - p0) / SL_W;
    const bool staged = len <= (uint32_t)HT_CAPL;
    const uint32_t *cp = staged ? reinterpret_cast<const uint32_t *>(base + (size_t)b * STG) + lane
                                : B.sl.col + p0 + lane;
    const AT *ap = staged ? reinterpret_cast<const AT *>(base + (size_t)b * STG + CB) + lane
                          : aw + p0 + lane;
    float m0 = 0.f, m1 = 0.f, m2 = 0.f;
    uint32_t e = 0;
    constexpr int U = 8;
    for (; e + U <= len; e += U) {
      uint32_t u[U];
      float wq[U];
#pragma unroll
      for (int j = 0; j < U; ++j) {
        u[j] = cp[(e + j) * SL_W];
        wq[j] = tofloat(ap[(e + j) * SL_W]);
      }
      float g0[U], g1[U], g2[U];
#pragma unroll
      for (int j = 0; j < U; ++j) ld3<CV>(src, u[j], g0[j], g1[j], g2[j]);
#pragma unroll
      for (int j = 0; j < U; ++j) {
        m0 += wq[j] * g0[j];
        m1 += wq[j] * g1[j];
        m2 += wq[j] * g2[j];
      }
    }
    for (; e < len; ++e) {
      const uint32_t u = cp[e * SL_W];
      const float wq = tofloat(ap[e * SL_W]);
      float g0, g1, g2;
      ld3<CV>(src, u, g0, g1, g2);
      m0 += wq * g0;
      m1 += wq * g1;
      m2 += wq * g2;
    }
    __syncwarp();
    if (v == SL_NONE) continue;
    if (first) {
      const float t0 = m0, t1 = m1, t2 = m2;
      m0 = G6[0] * t0 + G6[1] * t1 + G6[2] * t2;
      m1 = G6[3] * t0 + G6[4] * t1 + G6[5] * t2;
      m2 = G6[6] * t0 + G6[7] * t1 + G6[8] * t2;
    }
    float x0, x1, x2;
    ld3<CV>(B.xin, v, x0, x1, x2);
    const float w0 = m0 + G[0] * x0 + G[1] * x1 + G[2] * x2;
    const float w1 = m1 + G[3] * x0 + G[4] * x1 + G[5] * x2;
    const float w2 = m2 + G[6] * x0 + G[7] * x1 + G[8] * x2;
    if (FIN) {
      // w_0 as k_lrn_finish reads it: rounded to the evaluation's storage
      float a = w0, b = w1, c = w2;
      if (CV) cv_decode(cv_encode(w0, w1, w2), a, b, c);
      fin(v, a, b, c);
    } else {
      st3<CV>(dst, v, w0, w1, w2);
    }
  }
  fin_partials();
}

// The end of an application after the last Horner step wrote w_0:
// z = L^-T w_0 (z = L^-T x = D^-1 r after a fallback to block Jacobi) and
// the dot partials of the new z when part != null: r.r at part[0 .. np),
// r.z at part[np .. 2np), z.q at part[2np .. 3np) (np = gridDim.x) when
// want_rr / want_zq, else r.z alone at part[0 .. np).  A thread takes 4
// vertices at a time in vertex order (three float4 each of r, q and z, six
// of L^-1: r, q and z must be 16-byte aligned); the last n % 4 vertices go
// to thread 0 of block 0.
template <bool CV>
__global__ void __launch_bounds__(LG_T) k_lrn_finish(const SolveCtl *ctl, int gate, int32_t n,
                                                     const void *__restrict__ l6,
                                                     const void *__restrict__ xin,
                                                     const void *__restrict__ w0,
                                                     const float *__restrict__ r,
                                                     const float *__restrict__ q,
                                                     float *__restrict__ z,
                                                     double *__restrict__ part, int want_rr,
                                                     int want_zq) {
  __shared__ double sh[33];
  if (ctl && gate && ctl->status != ST_RUNNING) return;
  const bool fb = ctl && ctl->fallback;
  const void *w = fb ? xin : w0;
  DotAcc<float> rr, rz, zq;
  const int64_t nu = n / 4;
  const float4 *r4 = reinterpret_cast<const float4 *>(r);
  const float4 *q4 = reinterpret_cast<const float4 *>(q);
  float4 *z4 = reinterpret_cast<float4 *>(z);
  auto one = [&](const float *L, float a, float b, float c, float *zv) {
    // (L^-1)^T w, L^-1 = [[l0,0,0],[l1,l2,0],[l3,l4,l5]]
    zv[0] = L[0] * a + L[1] * b + L[3] * c;
    zv[1] = L[2] * b + L[4] * c;
    zv[2] = L[5] * c;
  };
  // four vertices: L^-1 in lv[24], z into zv[12], then the dot terms
  auto four = [&](int64_t v0, int cnt, const float *lv, bool vec) {
    float zv[12], rv[12], qv[12];
    for (int j = 0; j < cnt; ++j) {
      float a, b, c;
      ld3<CV>(w, (size_t)(v0 + j), a, b, c);
      one(lv + 6 * j, a, b, c, zv + 3 * j);
    }
    if (vec) {
#pragma unroll
      for (int k = 0; k < 3; ++k)
        z4[v0 / 4 * 3 + k] = make_float4(zv[4 * k], zv[4 * k + 1], zv[4 * k + 2], zv[4 * k + 3]);
    } else {
      for (int k = 0; k < cnt * 3; ++k) z[v0 * 3 + k] = zv[k];
    }
    if (!part) return;
    if (vec) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float4 a4 = r4[v0 / 4 * 3 + k];
        rv[4 * k] = a4.x; rv[4 * k + 1] = a4.y; rv[4 * k + 2] = a4.z; rv[4 * k + 3] = a4.w;
        if (want_zq) {
          const float4 b4 = q4[v0 / 4 * 3 + k];
          qv[4 * k] = b4.x; qv[4 * k + 1] = b4.y; qv[4 * k + 2] = b4.z; qv[4 * k + 3] = b4.w;
        }
      }
    } else {
      for (int k = 0; k < cnt * 3; ++k) {
        rv[k] = r[v0 * 3 + k];
        if (want_zq) qv[k] = q[v0 * 3 + k];
      }
    }
    for (int k = 0; k < cnt * 3; ++k) {
      if (want_rr) rr.add(rv[k], rv[k]);
      rz.add(rv[k], zv[k]);
      if (want_zq) zq.add(zv[k], qv[k]);
    }
  };
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nu;
       t += (int64_t)gridDim.x * blockDim.x) {
    float lv[24];
    ld_linv4<CV>(l6, t, lv);
    four(t * 4, 4, lv, true);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && nu * 4 < n) {
    // the last n % 4 vertices
    float lv[24];
    const int cnt = (int)(n - nu * 4);
    for (int j = 0; j < cnt; ++j) ld_linv<CV>(l6, (size_t)(nu * 4 + j), lv + 6 * j);
    four(nu * 4, cnt, lv, false);
  }
  if (!part) return;
  const double t1 = block_sum(rz.value(), sh);
  const double t0 = want_rr ? block_sum(rr.value(), sh) : 0.0;
  const double t2 = want_zq ? block_sum(zq.value(), sh) : 0.0;
  if (threadIdx.x == 0) {
    if (want_rr) part[blockIdx.x] = t0;
    part[(want_rr ? gridDim.x : 0) + blockIdx.x] = t1;
    if (want_zq) part[2 * gridDim.x + blockIdx.x] = t2;
  }
}

// x = L^-1 r for a fresh r (set-up, restarts and the standalone forward).
template <bool CV>
__global__ void k_lrn_xin(int32_t n, const void *__restrict__ l6, const float *__restrict__ r,
                          void *__restrict__ xin) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    float L[6];
    ld_linv<CV>(l6, (size_t)v, L);
    const float r0 = r[v * 3], r1 = r[v * 3 + 1], r2 = r[v * 3 + 2];
    st3<CV>(xin, v, L[0] * r0, L[1] * r0 + L[2] * r1, L[3] * r0 + L[4] * r1 + L[5] * r2);
  }
}

// K2 of the learned iteration: alpha = r.z / p.q; r -= alpha q; x = L^-1 r.
// x += alpha p is left to K3 (k_cg_direction_v4 with xupd), which decides
// the iteration from the partials k_lrn_finish leaves.  A thread takes 4
// vertices (three float4 of r and q, six of L^-1, four of x); the last
// n % 4 vertices go to thread 0 of the last CTA.
template <bool CV>
__global__ void __launch_bounds__(RED_T) k_lrn_update(SolveCtl *ctl, int par, int32_t n,
                                                      const double *__restrict__ part_in,
                                                      int np1, int pq_fin,
                                                      const float *__restrict__ q,
                                                      float *__restrict__ r,
                                                      const void *__restrict__ l6,
                                                      void *__restrict__ xin) {
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
  const int64_t nu = n / 4;
  const float4 *q4 = reinterpret_cast<const float4 *>(q);
  float4 *r4 = reinterpret_cast<float4 *>(r);
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
    ld_linv4<CV>(l6, u, lv);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      r4[u * 3 + k] = make_float4(rv[4 * k], rv[4 * k + 1], rv[4 * k + 2], rv[4 * k + 3]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float *L = lv + 6 * j, *R = rv + 3 * j;
      st3<CV>(xin, (size_t)(u * 4 + j), L[0] * R[0], L[1] * R[0] + L[2] * R[1],
              L[3] * R[0] + L[4] * R[1] + L[5] * R[2]);
    }
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    for (int64_t v = nu * 4; v < n; ++v) {
      float R[3];
      for (int k = 0; k < 3; ++k) {
        R[k] = r[v * 3 + k] - a * q[v * 3 + k];
        r[v * 3 + k] = R[k];
      }
      float L[6];
      ld_linv<CV>(l6, (size_t)v, L);
      st3<CV>(xin, (size_t)v, L[0] * R[0], L[1] * R[0] + L[2] * R[1],
              L[3] * R[0] + L[4] * R[1] + L[5] * R[2]);
    }
}

}  // namespace mpnn
}  // namespace sg
