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

// Three passes, each without a chain of dependent loads:
//   1. a thread per row finds its diagonal slot d (binary search of the
//      row's sorted columns) and writes fl(D + fl(s*K(d))) for the block to
//      scratch;
//   2. a flat, vectorised pass writes fl(0 + fl(s*K)) over every value;
//   3. a thread per row stores its scratch block into slot d.
// Pass 1 reads K before pass 2 may overwrite it, so out may alias K.
template <typename T, int BS>
__global__ void k_diag_terms(int32_t n, const uint32_t *__restrict__ rowptr,
                             const uint32_t *__restrict__ colidx, const T *__restrict__ D,
                             T ident, T s, const T *K, T *__restrict__ tmp,
                             uint32_t *__restrict__ dsl, int *err) {
  constexpr int B2 = BS * BS;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = rowptr[v], hi = rowptr[v + 1];
    const uint32_t e = hi;
    while (lo < hi) {
      const uint32_t m = lo + ((hi - lo) >> 1);
      if (colidx[m] < (uint32_t)v) lo = m + 1;
      else hi = m;
    }
    if (lo == e || colidx[lo] != (uint32_t)v) {
      atomicCAS(err, 0, (int)DEV_NO_DIAGONAL);
      dsl[v] = 0xffffffffu;
      continue;
    }
    dsl[v] = lo;
#pragma unroll
    for (int w = 0; w < B2; ++w) {
      const T base = D ? D[v * B2 + w] : ((w / BS == w % BS) ? ident : T(0));
      tmp[v * B2 + w] = rn_add(base, rn_mul(s, K[(int64_t)lo * B2 + w]));
    }
  }
}

template <typename T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4; };

template <typename T>
__global__ void k_scale_flat(int64_t len, T s, const T *K, T *out, int vec) {
  using V = typename Vec4<T>::type;
  const int64_t nv = vec ? len / 4 : 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
    V a = reinterpret_cast<const V *>(K)[i];
    a.x = rn_add(T(0), rn_mul(s, a.x));
    a.y = rn_add(T(0), rn_mul(s, a.y));
    a.z = rn_add(T(0), rn_mul(s, a.z));
    a.w = rn_add(T(0), rn_mul(s, a.w));
    reinterpret_cast<V *>(out)[i] = a;
  }
  for (int64_t i = nv * 4 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += stride)
    out[i] = rn_add(T(0), rn_mul(s, K[i]));
}

template <typename T, int BS>
__global__ void k_diag_store(int32_t n, const uint32_t *__restrict__ dsl,
                             const T *__restrict__ tmp, T *__restrict__ out) {
  constexpr int B2 = BS * BS;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t d = dsl[v];
    if (d == 0xffffffffu) continue;
#pragma unroll
    for (int w = 0; w < B2; ++w) out[(int64_t)d * B2 + w] = tmp[v * B2 + w];
  }
}

template <typename T, int BS>
int launch(Ctx *c, int32_t n, const uint32_t *rowptr, const uint32_t *colidx, int64_t nnzb,
           const void *D, double ident, double s, const void *K, void *out) {
  constexpr int B2 = BS * BS;
  const bool has_diag = D != nullptr || ident != 0.0;
  T *tmp = nullptr;
  uint32_t *dsl = nullptr;
  Scratch sc(c);
  if (has_diag) {
    SG_TRY(sc.reserve(Scratch::bytes_for((size_t)n * B2, sizeof(T)) +
                      Scratch::bytes_for((size_t)n, 4) + 512));
    tmp = sc.alloc<T>((size_t)n * B2);
    dsl = sc.alloc<uint32_t>((size_t)n);
    k_diag_terms<T, BS><<<grid_for(c, n, 256, 8), 256, 0, c->stream>>>(
        n, rowptr, colidx, (const T *)D, (T)ident, (T)s, (const T *)K, tmp, dsl, c->d_err);
    SG_CHECK_LAUNCH();
  }
  const int64_t len = nnzb * B2;
  const int vec = ((uintptr_t)K % 32 == 0 && (uintptr_t)out % 32 == 0) ? 1 : 0;
  if (len > 0) {
    k_scale_flat<T><<<grid_for(c, vec ? len / 4 + 1 : len, 256, 8), 256, 0, c->stream>>>(
        len, (T)s, (const T *)K, (T *)out, vec);
    SG_CHECK_LAUNCH();
  }
  if (has_diag) {
    k_diag_store<T, BS><<<grid_for(c, n, 256, 8), 256, 0, c->stream>>>(n, dsl, tmp, (T *)out);
    SG_CHECK_LAUNCH();
  }
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_bsr_add_diag(sg_ctx *h, int32_t n, int32_t bs, const uint32_t *rowptr,
                               const uint32_t *colidx, int64_t nnzb, int dtype,
                               const void *diag, double ident, double scale, const void *vals,
                               void *out) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_bsr_add_diag: null context");
  SG_REQUIRE(n >= 0 && bs >= 1 && bs <= 3, "sg_bsr_add_diag: n %d bs %d (bs 1..3)", n, bs);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_bsr_add_diag: dtype %d", dtype);
  SG_REQUIRE(diag == nullptr || ident == 0.0,
             "sg_bsr_add_diag: give either a diagonal array or ident, not both");
  SG_REQUIRE(nnzb >= 0, "sg_bsr_add_diag: nnzb %lld", (long long)nnzb);
  if (n == 0) return SG_OK;
  SG_REQUIRE(rowptr && colidx && (nnzb == 0 || (vals && out)), "sg_bsr_add_diag: null array");
#define SG_AD(BSV)                                                                          \
  if (bs == BSV)                                                                            \
    return dtype == SG_F64                                                                  \
               ? launch<double, BSV>(c, n, rowptr, colidx, nnzb, diag, ident, scale, vals, out) \
               : launch<float, BSV>(c, n, rowptr, colidx, nnzb, diag, ident, scale, vals, out);
  SG_AD(1) SG_AD(2) SG_AD(3)
#undef SG_AD
  return set_error(SG_ERR_UNSUPPORTED, "sg_bsr_add_diag: bs %d", bs);
}
