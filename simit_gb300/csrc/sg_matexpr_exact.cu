// System-matrix expressions on a blocked pattern: A = D + s*K, where D is a
// Diagonal-storage matrix (one bs x bs block per vertex, the result of a
// `map ... to points reduce +` whose target is the vertex set, src/storage.cpp:
// 358-360) or ident*I, and K an Indexed (blocked-CSR) matrix.  The result takes
// K's pattern, the higher-priority storage of the operands (src/storage.cpp:
// 416-470).  Operation order follows the lowered form of `MDK = MD + K`
// (apps/springs/isprings.sim:74): MDK = 0; MDK(l, l) = MD(l), stored through
// loc(l, l); then MDK(slot) = MDK(slot) + K(slot) for every slot of row l.  So
// a diagonal slot holds fl(D + fl(s*K)) and every other slot fl(0 + fl(s*K))
// (s = 1 leaves K unrounded).  This file is compiled with --fmad=false, and
// the products and sums are the explicitly rounded intrinsics, so no
// contraction changes a bit.
#include <stdint.h>

#include "sg_internal.cuh"

namespace sg {
namespace {

__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }

// G lanes per block row walk the row's nnz*BS*BS contiguous values, so a
// group's loads and stores are coalesced; the first U values of each lane are
// loaded with a fixed, predicated trip count so they are in flight together.
// Each lane notes whether it met the diagonal block; the group's OR tells
// whether the row has one.
template <typename T, int BS, int G>
__global__ void __launch_bounds__(256)
    k_add_diag(int32_t n, const uint32_t *__restrict__ rowptr,
               const uint32_t *__restrict__ colidx, const T *__restrict__ D, T ident,
               int has_diag, T s, const T *K, T *out, int *err) {
  constexpr int B2 = BS * BS;
  constexpr int U = (16 * B2 + G - 1) / G;  // rows of up to 16 blocks in one round
  const int lane = threadIdx.x % G;
  const unsigned mask = (G == 32) ? 0xffffffffu
                                  : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  const int64_t groups = (int64_t)gridDim.x * (blockDim.x / G);
  for (int64_t v = (int64_t)blockIdx.x * (blockDim.x / G) + threadIdx.x / G; v < n;
       v += groups) {
    const int64_t q0 = (int64_t)rowptr[v] * B2 + lane, q1 = (int64_t)rowptr[v + 1] * B2;
    unsigned found = 0;
    T kv[U];
    uint32_t cv[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int64_t q = q0 + (int64_t)k * G;
      if (q < q1) {
        kv[k] = K[q];
        cv[k] = colidx[q / B2];
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int64_t q = q0 + (int64_t)k * G;
      if (q < q1) {
        const int64_t slot = q / B2;
        const int w = (int)(q - slot * B2);
        const bool dg = cv[k] == (uint32_t)v;
        found |= dg ? 1u : 0u;
        T base = T(0);
        if (has_diag && dg) base = D ? D[v * B2 + w] : ((w / BS == w % BS) ? ident : T(0));
        out[q] = rn_add(base, rn_mul(s, kv[k]));
      }
    }
    for (int64_t q = q0 + (int64_t)U * G; q < q1; q += G) {
      const int64_t slot = q / B2;
      const int w = (int)(q - slot * B2);
      const bool dg = colidx[slot] == (uint32_t)v;
      found |= dg ? 1u : 0u;
      T base = T(0);
      if (has_diag && dg) base = D ? D[v * B2 + w] : ((w / BS == w % BS) ? ident : T(0));
      out[q] = rn_add(base, rn_mul(s, K[q]));
    }
    found = __reduce_or_sync(mask, found);
    if (has_diag && lane == 0 && !found) atomicCAS(err, 0, (int)DEV_NO_DIAGONAL);
  }
}

template <typename T, int BS>
int launch(Ctx *c, int32_t n, const uint32_t *rowptr, const uint32_t *colidx, const void *D,
           double ident, double s, const void *K, void *out) {
  constexpr int G = BS == 3 ? 32 : (BS == 2 ? 16 : 8);
  const int threads = 256;
  const int grid = grid_for(c, (int64_t)n * G, threads, 8);  // 64 warps per SM
  const int has_diag = (D != nullptr || ident != 0.0) ? 1 : 0;
  k_add_diag<T, BS, G><<<grid, threads, 0, c->stream>>>(
      n, rowptr, colidx, (const T *)D, (T)ident, has_diag, (T)s, (const T *)K, (T *)out,
      c->d_err);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_bsr_add_diag(sg_ctx *h, int32_t n, int32_t bs, const uint32_t *rowptr,
                               const uint32_t *colidx, int dtype, const void *diag,
                               double ident, double scale, const void *vals, void *out) {
  Ctx *c = as_ctx(h);
  SG_REQUIRE(c, "sg_bsr_add_diag: null context");
  SG_REQUIRE(n >= 0 && bs >= 1 && bs <= 3, "sg_bsr_add_diag: n %d bs %d (bs 1..3)", n, bs);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_bsr_add_diag: dtype %d", dtype);
  SG_REQUIRE(diag == nullptr || ident == 0.0,
             "sg_bsr_add_diag: give either a diagonal array or ident, not both");
  if (n == 0) return SG_OK;
  SG_REQUIRE(rowptr && colidx && vals && out, "sg_bsr_add_diag: null array");
#define SG_AD(BSV)                                                                          \
  if (bs == BSV)                                                                            \
    return dtype == SG_F64                                                                  \
               ? launch<double, BSV>(c, n, rowptr, colidx, diag, ident, scale, vals, out) \
               : launch<float, BSV>(c, n, rowptr, colidx, diag, ident, scale, vals, out);
  SG_AD(1) SG_AD(2) SG_AD(3)
#undef SG_AD
  return set_error(SG_ERR_UNSUPPORTED, "sg_bsr_add_diag: bs %d", bs);
}
