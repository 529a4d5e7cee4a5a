// Batched solves of many independent 3x3-blocked systems in one launch.
//
// The systems (e.g. 256 cloth sheets of uneven sizes) are concatenated into
// one block-diagonal matrix: system s owns block rows [sys_ptr[s],
// sys_ptr[s+1]) and its rows reference only its own columns.  A persistent
// kernel runs one whole PCG per CTA: CTAs take systems from a queue ordered
// largest first (longest-processing-time scheduling), and every phase of an
// iteration (SpMV, update, direction) is separated by __syncthreads only —
// systems never share data, so no grid-wide synchronisation exists.  The
// iteration is mixed precision: FP32 matrix and vectors, FP64 dot products,
// 3x3 block-Jacobi preconditioner; convergence (||r|| <= tol ||b||) is
// confirmed on the true residual b - A x accumulated in FP64, and a failed
// confirmation replaces r by it.  Every loop is bounded by maxiters.
//
// The reference solves each mesh with its own Simit program run (one harness
// kernel and a child kernel per loop, src/backend/gpu/gpu_function.cpp:
// 926-951); batching has no counterpart there.
#include <math.h>

#include <vector>

#include "sg_internal.cuh"
#include "sg_solver_kernels.cuh"

namespace sg {
namespace {

struct BatchArgs {
  int32_t nsys;
  const int32_t *sys_ptr;   // [nsys+1] block-row ranges
  const int32_t *order;     // [nsys] systems, largest first
  const uint32_t *rowptr, *colidx;
  const float *vals;
  const float *b;           // [n*3]
  float *x;                 // [n*3] in: guess, out: solution
  float *r, *p, *q, *z, *dinv;
  int *queue;               // work counter (zeroed before launch)
  int32_t *iters, *status;  // [nsys]
  double *relres;           // [nsys]
  double tol;
  int maxiters;
};

template <int G>
__device__ __forceinline__ double cta_sum(double v, double *sh) {
  // fixed-order block reduction (blockDim.x <= 1024)
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

// y = A x on rows [r0, r1) (G lanes per row); optional FP64 true residual
// y = b - A x accumulated in FP64 (x FP32) with partial of ||y||^2.
template <int G>
__device__ __forceinline__ double cta_spmv(const BatchArgs &a, int r0, int r1, const float *xv,
                                           float *y, bool residual, double *rr_out) {
  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = group_mask<G>();
  const int groups = blockDim.x / G;
  double acc = 0;
  for (int r = r0 + (int)(threadIdx.x / G); r < r1; r += groups) {
    const uint32_t e = a.rowptr[r + 1];
    if (residual) {  // FP64 accumulation (the true residual)
      double s0 = 0, s1 = 0, s2 = 0;
      for (uint32_t q = a.rowptr[r] + gl; q < e; q += G) {
        const uint32_t c = a.colidx[q];
        const float *v = a.vals + (size_t)q * 9;
        const float x0 = xv[c * 3], x1 = xv[c * 3 + 1], x2 = xv[c * 3 + 2];
        s0 += (double)v[0] * x0 + (double)v[1] * x1 + (double)v[2] * x2;
        s1 += (double)v[3] * x0 + (double)v[4] * x1 + (double)v[5] * x2;
        s2 += (double)v[6] * x0 + (double)v[7] * x1 + (double)v[8] * x2;
      }
      s0 = group_sum<G>(s0, mask);
      s1 = group_sum<G>(s1, mask);
      s2 = group_sum<G>(s2, mask);
      if (gl < 3) {
        const double val = (double)a.b[r * 3 + gl] - (gl == 0 ? s0 : (gl == 1 ? s1 : s2));
        acc += val * val;
        y[r * 3 + gl] = (float)val;
      }
    } else {  // the iteration's SpMV: FP32, as the single-system solver
      float s0 = 0, s1 = 0, s2 = 0;
      for (uint32_t q = a.rowptr[r] + gl; q < e; q += G) {
        const uint32_t c = a.colidx[q];
        const float *v = a.vals + (size_t)q * 9;
        const float x0 = xv[c * 3], x1 = xv[c * 3 + 1], x2 = xv[c * 3 + 2];
        s0 += v[0] * x0 + v[1] * x1 + v[2] * x2;
        s1 += v[3] * x0 + v[4] * x1 + v[5] * x2;
        s2 += v[6] * x0 + v[7] * x1 + v[8] * x2;
      }
      s0 = group_sum<G>(s0, mask);
      s1 = group_sum<G>(s1, mask);
      s2 = group_sum<G>(s2, mask);
      if (gl < 3) y[r * 3 + gl] = gl == 0 ? s0 : (gl == 1 ? s1 : s2);
    }
  }
  if (rr_out) *rr_out = acc;
  return acc;
}

template <int G>
__global__ void k_batched_pcg(BatchArgs a) {
  __shared__ double sh[34];
  __shared__ int sys_sh;
  for (;;) {
    if (threadIdx.x == 0) {
      const int k = atomicAdd(a.queue, 1);
      sys_sh = k < a.nsys ? a.order[k] : -1;
    }
    __syncthreads();
    const int s = sys_sh;
    __syncthreads();
    if (s < 0) break;
    const int r0 = a.sys_ptr[s], r1 = a.sys_ptr[s + 1];
    const int i0 = r0 * 3, i1 = r1 * 3;
    // block-Jacobi inverse of the diagonal blocks
    for (int v = r0 + threadIdx.x; v < r1; v += blockDim.x) {
      uint32_t lo = a.rowptr[v], hi = a.rowptr[v + 1];
      const uint32_t end = hi;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (a.colidx[mid] < (uint32_t)v) lo = mid + 1; else hi = mid;
      }
      float *D = a.dinv + (size_t)v * 9;
      if (lo >= end || a.colidx[lo] != (uint32_t)v) {
        for (int k = 0; k < 9; ++k) D[k] = 0.f;
        continue;
      }
      const float *m = a.vals + (size_t)lo * 9;
      const double c00 = (double)m[4] * m[8] - (double)m[5] * m[7];
      const double c01 = (double)m[5] * m[6] - (double)m[3] * m[8];
      const double c02 = (double)m[3] * m[7] - (double)m[4] * m[6];
      const double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
      if (!(fabs(det) > 0.0)) {
        for (int k = 0; k < 9; ++k) D[k] = 0.f;
        for (int k = 0; k < 3; ++k) D[k * 4] = m[k * 4] != 0.f ? 1.f / m[k * 4] : 0.f;
        continue;
      }
      const double id = 1.0 / det;
      D[0] = (float)(c00 * id);
      D[1] = (float)(((double)m[2] * m[7] - (double)m[1] * m[8]) * id);
      D[2] = (float)(((double)m[1] * m[5] - (double)m[2] * m[4]) * id);
      D[3] = (float)(c01 * id);
      D[4] = (float)(((double)m[0] * m[8] - (double)m[2] * m[6]) * id);
      D[5] = (float)(((double)m[2] * m[3] - (double)m[0] * m[5]) * id);
      D[6] = (float)(c02 * id);
      D[7] = (float)(((double)m[1] * m[6] - (double)m[0] * m[7]) * id);
      D[8] = (float)(((double)m[0] * m[4] - (double)m[1] * m[3]) * id);
    }
    // b'b
    double bb = 0;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) bb += (double)a.b[i] * a.b[i];
    bb = cta_sum<G>(bb, sh);
    const double tol2 = a.tol * a.tol * bb;
    // r = b - A x (FP64 accumulation)
    double rr = 0;
    cta_spmv<G>(a, r0, r1, a.x, a.r, true, &rr);
    rr = cta_sum<G>(rr, sh);
    int it = 0, st = 0;
    double rz = 0;
    auto precondition = [&]() {
      DotAcc<float> t;
      for (int v = r0 + threadIdx.x; v < r1; v += blockDim.x) {
        const float *D = a.dinv + (size_t)v * 9;
        const float q0 = a.r[v * 3], q1 = a.r[v * 3 + 1], q2 = a.r[v * 3 + 2];
        for (int k = 0; k < 3; ++k) {
          const float zk = D[k * 3] * q0 + D[k * 3 + 1] * q1 + D[k * 3 + 2] * q2;
          a.z[v * 3 + k] = zk;
          t.add(a.r[v * 3 + k], zk);
        }
      }
      return cta_sum<G>(t.value(), sh);
    };
    if (!(rr > tol2)) {
      st = SG_STATUS_CONVERGED;
    } else {
      rz = precondition();
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) a.p[i] = a.z[i];
      __syncthreads();
    }
    while (!st) {
      if (it >= a.maxiters) {
        st = SG_STATUS_MAXITER;
        break;
      }
      // q = A p, p.q
      cta_spmv<G>(a, r0, r1, a.p, a.q, false, nullptr);
      __syncthreads();
      DotAcc<float> pqa;
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) pqa.add(a.p[i], a.q[i]);
      const double pq = cta_sum<G>(pqa.value(), sh);
      if (!(pq > 0.0) || !isfinite(pq)) {
        st = isfinite(pq) ? SG_STATUS_BREAKDOWN : SG_STATUS_NAN;
        break;
      }
      const float al = (float)(rz / pq);
      DotAcc<float> rra;
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        a.x[i] += al * a.p[i];
        const float ri = a.r[i] - al * a.q[i];
        a.r[i] = ri;
        rra.add(ri, ri);
      }
      const double rrl = cta_sum<G>(rra.value(), sh);
      ++it;
      double rznew = precondition();
      if (rrl <= tol2) {
        // confirm on the true residual; replace r by it when it fails
        double rt = 0;
        __syncthreads();
        cta_spmv<G>(a, r0, r1, a.x, a.r, true, &rt);
        rt = cta_sum<G>(rt, sh);
        rr = rt;
        if (rt <= tol2) {
          st = SG_STATUS_CONVERGED;
          break;
        }
        rznew = precondition();
      }
      if (!isfinite(rznew)) {
        st = SG_STATUS_NAN;
        break;
      }
      const float be = (float)(rznew / rz);
      rz = rznew;
      for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) a.p[i] = a.z[i] + be * a.p[i];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      a.iters[s] = it;
      a.status[s] = st;
      a.relres[s] = bb > 0 ? sqrt(rr / bb) : 0.0;
    }
    __syncthreads();
  }
}

struct BatchCfg {
  int G, threads;
};
const BatchCfg kCfgs[] = {{4, 512}, {8, 512}, {4, 1024}, {8, 1024}, {4, 256}, {8, 256}};
constexpr int kNumCfgs = sizeof(kCfgs) / sizeof(kCfgs[0]);

int launch(Ctx *c, cudaStream_t st, const BatchArgs &a, int cfg) {
  const BatchCfg &k = kCfgs[cfg];
  const int per_sm = k.threads >= 1024 ? 2 : (k.threads >= 512 ? 4 : 8);
  int grid = c->num_sms * per_sm;
  if (grid > a.nsys) grid = a.nsys;
  if (grid < 1) grid = 1;
  SG_CHECK_CUDA(cudaMemsetAsync(a.queue, 0, sizeof(int), st));
  if (k.G == 4) k_batched_pcg<4><<<grid, k.threads, 0, st>>>(a);
  else k_batched_pcg<8><<<grid, k.threads, 0, st>>>(a);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_batched_pcg(sg_ctx *h, int32_t nsys, const int32_t *sys_ptr,
                              const int32_t *order, const sg_matrix *A, const float *b, float *x,
                              double tol, int32_t maxiters, int32_t config, int32_t *iters,
                              int32_t *status, double *relres) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && A && sys_ptr && order && b && x && iters && status && relres,
             "sg_batched_pcg: null argument");
  SG_REQUIRE(nsys >= 1 && A->bs == 3 && A->dtype == SG_F32 && A->n >= 1,
             "sg_batched_pcg: needs >= 1 system and an FP32 3x3-blocked matrix");
  SG_REQUIRE(config >= 0 && config < kNumCfgs, "sg_batched_pcg: config %d not in [0, %d)", config,
             kNumCfgs);
  SG_REQUIRE(maxiters >= 0 && tol > 0, "sg_batched_pcg: bad tol / maxiters");
  const int64_t len = (int64_t)A->n * 3;
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(len, 4) * 4 + Scratch::bytes_for(A->n * 9, 4) + 1024));
  BatchArgs a;
  a.nsys = nsys;
  a.sys_ptr = sys_ptr;
  a.order = order;
  a.rowptr = A->rowptr;
  a.colidx = A->colidx;
  a.vals = (const float *)A->vals;
  a.b = b;
  a.x = x;
  a.r = s.alloc<float>(len);
  a.p = s.alloc<float>(len);
  a.q = s.alloc<float>(len);
  a.z = s.alloc<float>(len);
  a.dinv = s.alloc<float>(A->n * 9);
  a.queue = s.alloc<int>(1);
  a.iters = iters;
  a.status = status;
  a.relres = relres;
  a.tol = tol;
  a.maxiters = maxiters;
  return launch(c, c->stream, a, config);
}

extern "C" int sg_batched_configs(void) { return kNumCfgs; }
