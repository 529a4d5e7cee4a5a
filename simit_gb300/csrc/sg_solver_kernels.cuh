// CG / PCG iteration kernels.
//
// The reference runs CG as user code (apps/springs/isprings.sim:77-93,
// apps/fem/fem_linear.sim:211-230, Jacobi-PCG apps/thermal/thermal.sim:
// 102-130): one SpMV, dots and axpys per iteration, each a separate loop; on
// its GPU backend every loop is a child kernel and every dot an atomic
// (src/backend/gpu/gpu_backend.cpp:335-365).  Here one iteration is three
// kernels with the dots fused in:
//   K1  q = A p                     + partial sums of p.q
//   K2  alpha = rz/pq; x += alpha p; r -= alpha q; z = M r
//                                   + partial sums of r.r, r.z (and z.q)
//   K3  beta; p = z + beta p; decide RUNNING / NEED_CHECK / MAXITER
// Every dot is an FP64 two-level sum: per-block partials in a fixed order,
// then each consumer block re-sums the partials in the same fixed order, so
// all blocks see identical scalars and results are run-to-run deterministic.
// Scalars that change per iteration live in two slots indexed by iteration
// parity, so no kernel reads a slot that another block of the same kernel
// writes.  A batch of iterations is captured once in a CUDA graph; kernels
// return immediately once the status leaves RUNNING.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sg_spmv.cuh"
#include "sg_tma.cuh"

namespace sg {

enum SolveStatus : int {
  ST_RUNNING = 0,
  ST_CONVERGED = 1,
  ST_MAXITER = 2,
  ST_BREAKDOWN = 3,
  ST_NAN = 4,
  ST_NEED_CHECK = 5,
};

struct SolveCtl {
  int status;
  int iter[2];        // iteration count, parity slots
  int maxiters;
  int check_every;    // > 0: NEED_CHECK every check_every iterations
  int flexible;       // Polak-Ribiere beta
  int fallback;       // learned preconditioner replaced by block Jacobi
  int pad;
  double rz[2];       // r.z of the current direction, parity slots
  double tol2;        // convergence threshold on r.r (iterated)
  double upd2;        // NEED_CHECK when r.r < upd2 (reliable update); 0 = off
  double last_rr;     // r.r at the last K3 (diagnostics)
  double last_alpha;
  // Last-CTA finalisation (see finalize_partials): K1's p.q total, and the
  // direction coefficient K2 decides for K3.  One slot each suffices: the
  // kernel that writes a slot never reads it, and stream order separates
  // the next write from the last read.
  double pq_tot;
  double beta;
  unsigned int tick1, tick2;
};

constexpr int RED_T = 256;

// Block-wide FP64 sum of one value per thread (fixed order), result to all.
__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) sh[32] = t;
  }
  __syncthreads();
  return sh[32];
}

// Sum of np partials (every block computes the same value).
__device__ __forceinline__ double sum_parts(const double *part, int np, double *sh) {
  double a = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) a += part[i];
  return block_sum(a, sh);
}

template <typename T> __device__ __forceinline__ bool finite_(T v) { return isfinite(v); }

// Last-CTA finalisation of per-CTA partial sums (nv arrays of gridDim.x
// values at part, part + gridDim.x, ...): every CTA stores its partials and
// takes a ticket; the CTA that takes the last ticket sums each array in index
// order (so the totals are deterministic), stores them in tot[0..nv) and
// re-arms the ticket.  Returns true in that CTA.  Called by all threads;
// nv <= 3.
__device__ __forceinline__ bool finalize_partials(const double *t, int nv, double *part,
                                                  unsigned int *ticket, double *tot,
                                                  double *sh) {
  __shared__ int last;
  if (threadIdx.x == 0) {
    for (int k = 0; k < nv; ++k) part[k * gridDim.x + blockIdx.x] = t[k];
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  // all nv arrays loaded in one pass (the last CTA works alone here, so its
  // load latency is the kernel's tail), then reduced one after the other
  double a[3] = {0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (k < nv) a[k] += __ldcg(part + k * gridDim.x + i);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (k >= nv) break;
    const double s = block_sum(a[k], sh);
    if (threadIdx.x == 0) tot[k] = s;
  }
  if (threadIdx.x == 0) *ticket = 0;
  return true;
}

// The control decision after K2's dots (shared by the finalising K2 and the
// reducing K3): iteration count, r.z slot, status, beta.  Executed by one
// thread; returns the new status.
__device__ __forceinline__ int cg_decide(SolveCtl *ctl, int par, double rr, double rznew,
                                         double zq, double alpha) {
  const double rzold = ctl->rz[par];
  const int it = ctl->iter[par] + 1;
  int st = ST_RUNNING;
  const bool lost = ctl->flexible && !ctl->fallback && !(rznew > 0.0);
  if (lost) st = ST_NEED_CHECK;  // z is no descent direction: fall back
  else if (!isfinite(rr) || !isfinite(rznew)) st = ST_NAN;
  else if (rr <= ctl->tol2) st = ST_NEED_CHECK;
  else if (ctl->upd2 > 0.0 && rr < ctl->upd2) st = ST_NEED_CHECK;
  else if (ctl->check_every > 0 && it % ctl->check_every == 0) st = ST_NEED_CHECK;
  else if (it >= ctl->maxiters) st = ST_MAXITER;
  ctl->iter[par ^ 1] = it;
  ctl->rz[par ^ 1] = rznew;
  ctl->last_rr = rr;
  if (lost) ctl->fallback = 1;
  // Fletcher-Reeves (the reference's beta = r'r_new / r'r_old, with z) or
  // Polak-Ribiere for a variable preconditioner: (z.r_new - z.r_old)/rz_old
  // where r_new - r_old = -alpha q.
  ctl->beta = ctl->flexible ? (-alpha * zq) / rzold : rznew / rzold;
  if (st != ST_RUNNING) ctl->status = st;
  return st;
}

// Per-thread dot-product accumulator.  FP64 arithmetic is scarce on this GPU
// (a few FP64 FMAs per SM per cycle), so the FP32 kernels accumulate their
// dot products as an unevaluated pair of floats: each product is split
// exactly into p + e with the FMA residual (TwoProduct) and added with
// Knuth's TwoSum, the compensated dot product "Dot2" of Ogita, Rump and
// Oishi (SIAM J. Sci. Comput. 26(6), 2005).  The pair carries about 48
// significant bits; value() converts it once to FP64, and the per-thread
// values are summed in FP64 from there on.  The intrinsics (_rn) are never
// contracted or reassociated by the compiler.  For FP64 operands the
// accumulator is a plain FP64 sum.
template <typename T> struct DotAcc;
template <> struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    const float s = __fadd_rn(hi, p);
    const float bv = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(p, bv));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(e, pe));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
template <> struct DotAcc<double> {
  double v = 0.0;
  __device__ __forceinline__ void add(double a, double b) { v += a * b; }
  __device__ __forceinline__ double value() const { return v; }
};

// K1: q = A p, partial p.q.  BS = 3 or 1 (G lanes per row), 0 = any bs.
template <int BS, int G, typename MT, typename VT>
__global__ void __launch_bounds__(RED_T) k_cg_spmv(const SolveCtl *__restrict__ ctl, int32_t n,
                                                   int32_t bs, const uint32_t *__restrict__ rowptr,
                                                   const uint32_t *__restrict__ colidx,
                                                   const MT *__restrict__ vals,
                                                   const VT *__restrict__ p, VT *__restrict__ q,
                                                   double *__restrict__ part) {
  __shared__ double sh[33];
  if (ctl->status != ST_RUNNING) return;
  double acc = 0;
  if (BS == 3 || BS == 1) {
    const int gl = threadIdx.x & (G - 1);
    const unsigned mask = group_mask<G>();
    const int64_t stride = (int64_t)gridDim.x * (blockDim.x / G);
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; r < n; r += stride) {
      if (BS == 3) {
        VT y0, y1, y2;
        bsr3_row<G, MT, VT, VT>(rowptr, colidx, vals, p, r, gl, mask, y0, y1, y2);
        if (gl == 0) {
          q[r * 3 + 0] = y0; q[r * 3 + 1] = y1; q[r * 3 + 2] = y2;
          acc += (double)p[r * 3 + 0] * (double)y0 + (double)p[r * 3 + 1] * (double)y1 +
                 (double)p[r * 3 + 2] * (double)y2;
        }
      } else {
        VT y = csr_row<G, MT, VT, VT>(rowptr, colidx, vals, p, r, gl, mask);
        if (gl == 0) {
          q[r] = y;
          acc += (double)p[r] * (double)y;
        }
      }
    }
  } else {
    for (int64_t qq = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; qq < n;
         qq += (int64_t)gridDim.x * blockDim.x) {
      for (int q1 = 0; q1 < bs; ++q1) {
        VT s = 0;
        for (uint32_t qp = rowptr[qq]; qp < rowptr[qq + 1]; ++qp) {
          const int64_t c = colidx[qp];
          VT t = 0;
          for (int p1 = 0; p1 < bs; ++p1)
            t += (VT)vals[(size_t)qp * bs * bs + q1 * bs + p1] * p[c * bs + p1];
          s += t;
        }
        q[qq * bs + q1] = s;
        acc += (double)p[qq * bs + q1] * (double)s;
      }
    }
  }
  double tot = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// Preconditioner kinds applied inside K2.
enum PrecKind : int { PK_NONE = 0, PK_JACOBI = 1, PK_BLOCK3 = 2, PK_EXTERNAL = 3 };

// K2: alpha, x/r update, z = M r, partials of r.r, r.z, z.q.
// part_in: np1 partials of p.q; part_out: 3 * gridDim.x (rr | rz | zq).
template <typename VT, typename XT, int PREC>
__global__ void __launch_bounds__(RED_T) k_cg_update(SolveCtl *ctl, int par, int64_t len,
                                                     const double *__restrict__ part_in, int np1,
                                                     const VT *__restrict__ p,
                                                     const VT *__restrict__ q, VT *__restrict__ r,
                                                     XT *__restrict__ x, VT *__restrict__ z,
                                                     const VT *__restrict__ dinv,
                                                     double *__restrict__ part_out) {
  __shared__ double sh[33];
  if (ctl->status != ST_RUNNING) return;
  const double pq = sum_parts(part_in, np1, sh);
  const double rz = ctl->rz[par];
  if (!(pq > 0.0) || !isfinite(pq)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
    return;
  }
  const double alpha = rz / pq;
  const VT a = (VT)alpha;
  double rr = 0, rzs = 0, zq = 0;
  if (PREC == PK_BLOCK3) {
    // 3x3 block-Jacobi: dinv holds 9 values per vertex; one thread per vertex
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v * 3 < len;
         v += (int64_t)gridDim.x * blockDim.x) {
      VT rv[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int64_t i = v * 3 + k;
        x[i] = (XT)(x[i] + (XT)(a * p[i]));
        rv[k] = r[i] - a * q[i];
        r[i] = rv[k];
      }
      const VT *D = dinv + v * 9;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const VT zk = D[k * 3] * rv[0] + D[k * 3 + 1] * rv[1] + D[k * 3 + 2] * rv[2];
        z[v * 3 + k] = zk;
        rr += (double)rv[k] * (double)rv[k];
        rzs += (double)rv[k] * (double)zk;
        zq += (double)zk * (double)q[v * 3 + k];
      }
    }
  } else {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
      const VT pi = p[i], qi = q[i];
      x[i] = (XT)(x[i] + (XT)(a * pi));
      const VT ri = r[i] - a * qi;
      r[i] = ri;
      VT zi = ri;
      if (PREC == PK_JACOBI) zi = dinv[i] * ri;
      if (PREC != PK_EXTERNAL) {
        if (PREC != PK_NONE) z[i] = zi;
        rzs += (double)ri * (double)zi;
        zq += (double)zi * (double)qi;
      }
      rr += (double)ri * (double)ri;
    }
  }
  const double t0 = block_sum(rr, sh);
  const double t1 = block_sum(rzs, sh);
  const double t2 = block_sum(zq, sh);
  if (threadIdx.x == 0) {
    part_out[blockIdx.x] = t0;
    part_out[gridDim.x + blockIdx.x] = t1;
    part_out[2 * gridDim.x + blockIdx.x] = t2;
    if (blockIdx.x == 0) ctl->last_alpha = alpha;
  }
}

// K3: beta, direction update, control decisions.
// part_in: 3 * np2 partials (rr | rz | zq) from K2 (or from the external
// preconditioner's dot kernel).
template <typename VT>
__global__ void __launch_bounds__(RED_T) k_cg_direction(SolveCtl *ctl, int par, int64_t len,
                                                        const double *__restrict__ part_in,
                                                        int np2, const VT *__restrict__ z,
                                                        VT *__restrict__ p) {
  __shared__ double sh[33];
  if (ctl->status != ST_RUNNING) return;
  const double rr = sum_parts(part_in, np2, sh);
  const double rznew = sum_parts(part_in + np2, np2, sh);
  const double zq = sum_parts(part_in + 2 * np2, np2, sh);
  const double rzold = ctl->rz[par];
  const int it = ctl->iter[par] + 1;
  int st = ST_RUNNING;
  const bool lost = ctl->flexible && !ctl->fallback && !(rznew > 0.0);
  if (lost) st = ST_NEED_CHECK;  // z is no descent direction: fall back
  else if (!isfinite(rr) || !isfinite(rznew)) st = ST_NAN;
  else if (rr <= ctl->tol2) st = ST_NEED_CHECK;
  else if (ctl->upd2 > 0.0 && rr < ctl->upd2) st = ST_NEED_CHECK;
  else if (ctl->check_every > 0 && it % ctl->check_every == 0) st = ST_NEED_CHECK;
  else if (it >= ctl->maxiters) st = ST_MAXITER;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->iter[par ^ 1] = it;
    ctl->rz[par ^ 1] = rznew;
    ctl->last_rr = rr;
    if (lost) ctl->fallback = 1;
    if (st != ST_RUNNING) ctl->status = st;
  }
  if (st != ST_RUNNING) return;
  // Fletcher-Reeves (the reference's beta = r'r_new / r'r_old, with z) or
  // Polak-Ribiere for a variable preconditioner: (z.r_new - z.r_old)/rz_old
  // where r_new - r_old = -alpha q.
  double beta;
  if (ctl->flexible) beta = (-ctl->last_alpha * zq) / rzold;
  else beta = rznew / rzold;
  const VT b = (VT)beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + b * p[i];
}

// ---------------------------------------------------------------------------
// FP32 (mixed-precision) K2 / K3 with 16-byte loads and stores.  One thread
// takes four vertices at a time: three float4 of each vector and nine of the
// block-Jacobi inverse, all contiguous across the warp.  The buffers are
// cudaMalloc'd (256-byte aligned); the last len % 12 (or len % 4) entries go
// through the scalar loop of thread 0 of the last block.  Same partial sums
// as the scalar kernels, in a different (fixed) order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void ld4(const float *p, int64_t i, float *o) {
  const float4 v = reinterpret_cast<const float4 *>(p)[i];
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void st4(float *p, int64_t i, const float *o) {
  reinterpret_cast<float4 *>(p)[i] = make_float4(o[0], o[1], o[2], o[3]);
}

// pq_fin: K1 left the p.q total in ctl->pq_tot (else the np1 partials are
// summed here).  FIN (not with an external preconditioner, whose dots come
// after K2): the last CTA sums r.r, r.z, z.q and takes K3's decision.
template <int PREC, bool FIN>
__global__ void __launch_bounds__(RED_T, 3) k_cg_update_v4(SolveCtl *ctl, int par, int64_t len,
                                                        const double *__restrict__ part_in,
                                                        int np1, int pq_fin,
                                                        const float *__restrict__ p,
                                                        const float *__restrict__ q,
                                                        float *__restrict__ r,
                                                        float *__restrict__ x,
                                                        float *__restrict__ z,
                                                        const float *__restrict__ dinv,
                                                        double *__restrict__ part_out) {
  // FP32 block Jacobi runs k_cg_update_w, whose inverse blocks are packed
  static_assert(PREC != PK_BLOCK3, "FP32 block Jacobi: use k_cg_update_w");
  __shared__ double sh[33];
  if (ctl->status != ST_RUNNING) return;
  const double pq = pq_fin ? ctl->pq_tot : sum_parts(part_in, np1, sh);
  const double rz = ctl->rz[par];
  if (!(pq > 0.0) || !isfinite(pq)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
    return;
  }
  const double alpha = rz / pq;
  const float a = (float)alpha;
  DotAcc<float> rr, rzs, zq;
  constexpr int W = PREC == PK_BLOCK3 ? 12 : 4;  // floats per thread step
  constexpr int NV = W / 4;                      // float4 per vector
  const int64_t nu = len / W;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nu;
       u += (int64_t)gridDim.x * blockDim.x) {
    float pv[W], qv[W], rv[W], xv[W], zv[W];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      ld4(p, u * NV + k, pv + 4 * k);
      ld4(q, u * NV + k, qv + 4 * k);
      ld4(r, u * NV + k, rv + 4 * k);
      ld4(x, u * NV + k, xv + 4 * k);
    }
    float dv[PREC == PK_BLOCK3 ? 36 : (PREC == PK_JACOBI ? 4 : 1)];
    if (PREC == PK_BLOCK3) {
#pragma unroll
      for (int k = 0; k < 9; ++k) ld4(dinv, u * 9 + k, dv + 4 * k);
    } else if (PREC == PK_JACOBI) {
      ld4(dinv, u, dv);
    }
#pragma unroll
    for (int k = 0; k < W; ++k) {
      xv[k] = xv[k] + a * pv[k];
      rv[k] = rv[k] - a * qv[k];
    }
    if (PREC == PK_BLOCK3) {
#pragma unroll
      for (int v = 0; v < 4; ++v)
#pragma unroll
        for (int k = 0; k < 3; ++k)
          zv[v * 3 + k] = dv[v * 9 + k * 3] * rv[v * 3] + dv[v * 9 + k * 3 + 1] * rv[v * 3 + 1] +
                          dv[v * 9 + k * 3 + 2] * rv[v * 3 + 2];
    } else {
#pragma unroll
      for (int k = 0; k < W; ++k) zv[k] = PREC == PK_JACOBI ? dv[k] * rv[k] : rv[k];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      st4(x, u * NV + k, xv + 4 * k);
      st4(r, u * NV + k, rv + 4 * k);
      if (PREC == PK_BLOCK3 || PREC == PK_JACOBI) st4(z, u * NV + k, zv + 4 * k);
    }
#pragma unroll
    for (int k = 0; k < W; ++k) {
      rr.add(rv[k], rv[k]);
      if (PREC != PK_EXTERNAL) {
        rzs.add(rv[k], zv[k]);
        zq.add(zv[k], qv[k]);
      }
    }
  }
  // tail: the last len % W entries, scalar, by one thread
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    for (int64_t i0 = nu * W; i0 < len; i0 += (PREC == PK_BLOCK3 ? 3 : 1)) {
      const int m = PREC == PK_BLOCK3 ? 3 : 1;
      float rv[3], zv[3];
      for (int k = 0; k < m; ++k) {
        const int64_t i = i0 + k;
        x[i] = x[i] + a * p[i];
        rv[k] = r[i] - a * q[i];
        r[i] = rv[k];
      }
      for (int k = 0; k < m; ++k) {
        const int64_t i = i0 + k;
        if (PREC == PK_BLOCK3) {
          const float *D = dinv + (i0 / 3) * 9;
          zv[k] = D[k * 3] * rv[0] + D[k * 3 + 1] * rv[1] + D[k * 3 + 2] * rv[2];
        } else {
          zv[k] = PREC == PK_JACOBI ? dinv[i] * rv[k] : rv[k];
        }
        if (PREC == PK_BLOCK3 || PREC == PK_JACOBI) z[i] = zv[k];
        rr.add(rv[k], rv[k]);
        if (PREC != PK_EXTERNAL) {
          rzs.add(rv[k], zv[k]);
          zq.add(zv[k], q[i]);
        }
      }
    }
  }
  const double t[3] = {block_sum(rr.value(), sh), block_sum(rzs.value(), sh),
                       block_sum(zq.value(), sh)};
  if (FIN) {
    double tot[3];  // written and read by thread 0 of the last CTA
    if (finalize_partials(t, 3, part_out, &ctl->tick2, tot, sh) && threadIdx.x == 0) {
      ctl->last_alpha = alpha;
      cg_decide(ctl, par, tot[0], tot[1], tot[2], alpha);
    }
  } else if (threadIdx.x == 0) {
    part_out[blockIdx.x] = t[0];
    part_out[gridDim.x + blockIdx.x] = t[1];
    part_out[2 * gridDim.x + blockIdx.x] = t[2];
    if (blockIdx.x == 0) ctl->last_alpha = alpha;
  }
}

// K2 for FP32 vectors and 3x3 block Jacobi with warp-staged, fully coalesced
// accesses.  A warp takes 128 vertices at a time: it loads the chunk of
// p, q, r, x (96 float4 each) and of the packed symmetric D^-1 (6 values per
// vertex, k_diag_inv PACK6: 192 float4) with lane-consecutive
// 16-byte loads into its shared-memory slice, each lane then reads its four
// vertices (3 and 9 consecutive float4, conflict-free), and the results go
// back through shared memory to lane-consecutive stores.  Same arithmetic,
// partial sums and finalisation as k_cg_update_v4<PK_BLOCK3>.  The last
// len % 12 entries are done by the scalar tail of thread 0 of the last CTA.
constexpr int K2W_WARPS = 8;
struct K2WarpSmem {
  float4 p[96], q[96], r[96], x[96], d[192];
};

// XUPD = false: x += alpha p is left to K3 (k_cg_direction_v4 with xupd), so
// this kernel neither reads p and x nor writes x.
template <bool FIN, bool XUPD = true>
__global__ void __launch_bounds__(K2W_WARPS * 32) k_cg_update_w(
    SolveCtl *ctl, int par, int64_t len, const double *__restrict__ part_in, int np1,
    int pq_fin, const float *__restrict__ p, const float *__restrict__ q, float *__restrict__ r,
    float *__restrict__ x, float *__restrict__ z, const float *__restrict__ dinv,
    double *__restrict__ part_out) {
  extern __shared__ __align__(16) unsigned char k2w_raw[];
  __shared__ double sh[33];
  pdl_wait_and_release();
  if (ctl->status != ST_RUNNING) return;
  const double pq = pq_fin ? ctl->pq_tot : sum_parts(part_in, np1, sh);
  const double rz = ctl->rz[par];
  if (!(pq > 0.0) || !isfinite(pq)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->status = isfinite(pq) ? ST_BREAKDOWN : ST_NAN;
    return;
  }
  const double alpha = rz / pq;
  const float a = (float)alpha;
  const int lane = threadIdx.x & 31;
  K2WarpSmem &w = reinterpret_cast<K2WarpSmem *>(k2w_raw)[threadIdx.x >> 5];
  const float4 *p4 = reinterpret_cast<const float4 *>(p);
  const float4 *q4 = reinterpret_cast<const float4 *>(q);
  float4 *r4 = reinterpret_cast<float4 *>(r);
  float4 *x4 = reinterpret_cast<float4 *>(x);
  float4 *z4 = reinterpret_cast<float4 *>(z);
  const float4 *d4 = reinterpret_cast<const float4 *>(dinv);
  const int64_t nu = len / 12;          // complete 4-vertex units
  const int64_t nf = nu * 3;            // their float4 of each vector
  const int64_t nchunks = (nu + 31) / 32;
  DotAcc<float> rr, rzs, zq;
  for (int64_t c = (int64_t)blockIdx.x * K2W_WARPS + (threadIdx.x >> 5); c < nchunks;
       c += (int64_t)gridDim.x * K2W_WARPS) {
    const int64_t f0 = c * 96, d0 = c * 192;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int64_t f = f0 + lane + 32 * j;
      if (f < nf) {
        if (XUPD) w.p[lane + 32 * j] = p4[f];
        w.q[lane + 32 * j] = q4[f];
        w.r[lane + 32 * j] = r4[f];
        if (XUPD) w.x[lane + 32 * j] = x4[f];
      }
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const int64_t f = d0 + lane + 32 * j;
      if (f < nf * 2) w.d[lane + 32 * j] = d4[f];
    }
    __syncwarp();
    const bool mine = c * 32 + lane < nu;
    float pv[12], qv[12], rv[12], xv[12], zv[12], dv[24];
    if (mine) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float4 b4 = w.q[3 * lane + j], c4 = w.r[3 * lane + j];
        qv[4 * j] = b4.x; qv[4 * j + 1] = b4.y; qv[4 * j + 2] = b4.z; qv[4 * j + 3] = b4.w;
        rv[4 * j] = c4.x; rv[4 * j + 1] = c4.y; rv[4 * j + 2] = c4.z; rv[4 * j + 3] = c4.w;
        if (XUPD) {
          const float4 a4 = w.p[3 * lane + j], e4 = w.x[3 * lane + j];
          pv[4 * j] = a4.x; pv[4 * j + 1] = a4.y; pv[4 * j + 2] = a4.z; pv[4 * j + 3] = a4.w;
          xv[4 * j] = e4.x; xv[4 * j + 1] = e4.y; xv[4 * j + 2] = e4.z; xv[4 * j + 3] = e4.w;
        }
      }
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        const float4 g4 = w.d[6 * lane + j];
        dv[4 * j] = g4.x; dv[4 * j + 1] = g4.y; dv[4 * j + 2] = g4.z; dv[4 * j + 3] = g4.w;
      }
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        if (XUPD) xv[k] = xv[k] + a * pv[k];
        rv[k] = rv[k] - a * qv[k];
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {  // symmetric inverse, upper triangle
        const float *m = dv + v * 6, *rq = rv + v * 3;
        zv[v * 3 + 0] = m[0] * rq[0] + m[1] * rq[1] + m[2] * rq[2];
        zv[v * 3 + 1] = m[1] * rq[0] + m[3] * rq[1] + m[4] * rq[2];
        zv[v * 3 + 2] = m[2] * rq[0] + m[4] * rq[1] + m[5] * rq[2];
      }
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        rr.add(rv[k], rv[k]);
        rzs.add(rv[k], zv[k]);
        zq.add(zv[k], qv[k]);
      }
    }
    __syncwarp();  // every lane has read its inputs
    if (mine) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        if (XUPD)
          w.x[3 * lane + j] = make_float4(xv[4 * j], xv[4 * j + 1], xv[4 * j + 2], xv[4 * j + 3]);
        w.r[3 * lane + j] = make_float4(rv[4 * j], rv[4 * j + 1], rv[4 * j + 2], rv[4 * j + 3]);
        w.p[3 * lane + j] = make_float4(zv[4 * j], zv[4 * j + 1], zv[4 * j + 2], zv[4 * j + 3]);
      }
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int64_t f = f0 + lane + 32 * j;
      if (f < nf) {
        if (XUPD) x4[f] = w.x[lane + 32 * j];
        r4[f] = w.r[lane + 32 * j];
        z4[f] = w.p[lane + 32 * j];
      }
    }
    __syncwarp();  // the slice is refilled by the next chunk
  }
  // tail: the last len % 12 entries, scalar, by one thread
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
    for (int64_t i0 = nu * 12; i0 < len; i0 += 3) {
      float rv[3];
      for (int k = 0; k < 3; ++k) {
        const int64_t i = i0 + k;
        if (XUPD) x[i] = x[i] + a * p[i];
        rv[k] = r[i] - a * q[i];
        r[i] = rv[k];
      }
      const float *m = dinv + (i0 / 3) * 6;
      const float zz[3] = {m[0] * rv[0] + m[1] * rv[1] + m[2] * rv[2],
                           m[1] * rv[0] + m[3] * rv[1] + m[4] * rv[2],
                           m[2] * rv[0] + m[4] * rv[1] + m[5] * rv[2]};
      for (int k = 0; k < 3; ++k) {
        const float zk = zz[k];
        z[i0 + k] = zk;
        rr.add(rv[k], rv[k]);
        rzs.add(rv[k], zk);
        zq.add(zk, q[i0 + k]);
      }
    }
  }
  const double t[3] = {block_sum(rr.value(), sh), block_sum(rzs.value(), sh),
                       block_sum(zq.value(), sh)};
  if (FIN) {
    double tot[3];
    if (finalize_partials(t, 3, part_out, &ctl->tick2, tot, sh) && threadIdx.x == 0) {
      ctl->last_alpha = alpha;
      cg_decide(ctl, par, tot[0], tot[1], tot[2], alpha);
    }
  } else if (threadIdx.x == 0) {
    part_out[blockIdx.x] = t[0];
    part_out[gridDim.x + blockIdx.x] = t[1];
    part_out[2 * gridDim.x + blockIdx.x] = t[2];
    if (blockIdx.x == 0) ctl->last_alpha = alpha;
  }
}

// K3 for FP32 vectors: the control decisions of k_cg_direction, then
// p = z + beta p with float4 accesses.
// fin: K2 already took the decision and left beta in ctl->beta.
// xupd: K2 left x += alpha p to this kernel, which applies it with the
// direction it is about to replace; when K2 (fin) or this kernel (!fin)
// stopped the batch, the host applies that last update instead (the early
// returns below).
static __global__ void __launch_bounds__(RED_T) k_cg_direction_v4(SolveCtl *ctl, int par, int64_t len,
                                                           const double *__restrict__ part_in,
                                                           int np2, int fin,
                                                           const float *__restrict__ z,
                                                           float *__restrict__ p,
                                                           float *__restrict__ x, int xupd) {
  __shared__ double sh[33];
  pdl_wait_and_release();
  if (ctl->status != ST_RUNNING) return;
  if (fin) {
    const float b = (float)ctl->beta;
    const float a = (float)ctl->last_alpha;
    const int64_t nu = len / 4;
    for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nu;
         u += (int64_t)gridDim.x * blockDim.x) {
      float zv[4], pv[4];
      ld4(z, u, zv);
      ld4(p, u, pv);
      if (xupd) {
        float xv[4];
        ld4(x, u, xv);
#pragma unroll
        for (int k = 0; k < 4; ++k) xv[k] = xv[k] + a * pv[k];
        st4(x, u, xv);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) pv[k] = zv[k] + b * pv[k];
      st4(p, u, pv);
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
      for (int64_t i = nu * 4; i < len; ++i) {
        if (xupd) x[i] = x[i] + a * p[i];
        p[i] = z[i] + b * p[i];
      }
    return;
  }
  const double rr = sum_parts(part_in, np2, sh);
  const double rznew = sum_parts(part_in + np2, np2, sh);
  const double zq = sum_parts(part_in + 2 * np2, np2, sh);
  const double rzold = ctl->rz[par];
  const int it = ctl->iter[par] + 1;
  int st = ST_RUNNING;
  const bool lost = ctl->flexible && !ctl->fallback && !(rznew > 0.0);
  if (lost) st = ST_NEED_CHECK;
  else if (!isfinite(rr) || !isfinite(rznew)) st = ST_NAN;
  else if (rr <= ctl->tol2) st = ST_NEED_CHECK;
  else if (ctl->upd2 > 0.0 && rr < ctl->upd2) st = ST_NEED_CHECK;
  else if (ctl->check_every > 0 && it % ctl->check_every == 0) st = ST_NEED_CHECK;
  else if (it >= ctl->maxiters) st = ST_MAXITER;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->iter[par ^ 1] = it;
    ctl->rz[par ^ 1] = rznew;
    ctl->last_rr = rr;
    if (lost) ctl->fallback = 1;
    if (st != ST_RUNNING) ctl->status = st;
  }
  if (st != ST_RUNNING) return;
  const double beta = ctl->flexible ? (-ctl->last_alpha * zq) / rzold : rznew / rzold;
  const float b = (float)beta;
  // xupd: the iteration's x += alpha p, applied here with the direction it
  // is about to replace (on a stop above the host applies it instead)
  const float a = (float)ctl->last_alpha;
  const int64_t nu = len / 4;
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < nu;
       u += (int64_t)gridDim.x * blockDim.x) {
    float zv[4], pv[4];
    ld4(z, u, zv);
    ld4(p, u, pv);
    if (xupd) {
      float xv[4];
      ld4(x, u, xv);
#pragma unroll
      for (int k = 0; k < 4; ++k) xv[k] = xv[k] + a * pv[k];
      st4(x, u, xv);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) pv[k] = zv[k] + b * pv[k];
    st4(p, u, pv);
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    for (int64_t i = nu * 4; i < len; ++i) {
      if (xupd) x[i] = x[i] + a * p[i];
      p[i] = z[i] + b * p[i];
    }
}

// ---------------------------------------------------------------------------
// Set-up / check kernels
// ---------------------------------------------------------------------------

// FP32 -> FP64 without the FP64 unit, which does the residual's
// multiply-adds and is scarce on this GPU (about 2 per SM and clock): the
// sign, the exponent rebiased by 1023 - 127 and the mantissa moved up 29
// bits; subnormals normalised by their leading zeros; inf and NaN keep
// their payload.  Exact, as the conversion is.
__device__ __forceinline__ double widen_f32(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t m = u & 0x7fffffffu, e8 = m >> 23;
  uint64_t mag;
  if (e8 == 0) {
    const int k = __clz(m);  // m > 0: k in [9, 31]
    mag = m == 0 ? 0ull
                 : ((uint64_t)(905 - k) << 52) | ((uint64_t)((m << (k - 8)) & 0x7fffffu) << 29);
  } else if (e8 == 255) {
    mag = (0x7ffull << 52) | ((uint64_t)(m & 0x7fffffu) << 29);
  } else {
    mag = ((uint64_t)m + (896ull << 23)) << 29;
  }
  return __longlong_as_double((long long)(((uint64_t)(u & 0x80000000u) << 32) | mag));
}

// y_row = sum of the row's FP32 3x3 blocks times FP64 x, accumulated in
// FP64 by one multiply-add per entry (9 per block) on widened entries; a
// lane's even and odd blocks go to separate sums, which halves the chains
// of dependent multiply-adds.
template <int G>
__device__ __forceinline__ void bsr3_row_widen(const uint32_t *__restrict__ rowptr,
                                               const uint32_t *__restrict__ colidx,
                                               const float *__restrict__ vals,
                                               const double *__restrict__ x, int64_t row, int gl,
                                               unsigned mask, double &y0, double &y1,
                                               double &y2) {
  const uint32_t e = ldg(rowptr + row + 1);
  uint32_t b = ldg(rowptr + row) + gl;
  double a[2][3] = {{0, 0, 0}, {0, 0, 0}};
  auto block = [&](uint32_t k, double *acc) {
    const uint32_t c = ldg(colidx + k);
    const float *v = vals + (size_t)k * 9;
    const double x0 = ldg(x + (size_t)c * 3 + 0);
    const double x1 = ldg(x + (size_t)c * 3 + 1);
    const double x2 = ldg(x + (size_t)c * 3 + 2);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      acc[i] = fma(widen_f32(ld_stream(v + 3 * i + 0)), x0, acc[i]);
      acc[i] = fma(widen_f32(ld_stream(v + 3 * i + 1)), x1, acc[i]);
      acc[i] = fma(widen_f32(ld_stream(v + 3 * i + 2)), x2, acc[i]);
    }
  };
  for (; b + G < e; b += 2 * G) {
    block(b, a[0]);
    block(b + G, a[1]);
  }
  if (b < e) block(b, a[0]);
  y0 = group_sum<G>(a[0][0] + a[1][0], mask);
  y1 = group_sum<G>(a[0][1] + a[1][1], mask);
  y2 = group_sum<G>(a[0][2] + a[1][2], mask);
}

// r_hi = b - A x_hi with FP64 accumulation (matrix MT, x FP64).
template <int G, typename MT>
__global__ void __launch_bounds__(RED_T) k_true_residual3(int32_t n,
                                                          const uint32_t *__restrict__ rowptr,
                                                          const uint32_t *__restrict__ colidx,
                                                          const MT *__restrict__ vals,
                                                          const double *__restrict__ x,
                                                          const double *__restrict__ b,
                                                          double *__restrict__ rhi,
                                                          double *__restrict__ part) {
  __shared__ double sh[33];
  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = group_mask<G>();
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x / G);
  double acc = 0;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; r < n; r += stride) {
    double y0, y1, y2;
    if constexpr (sizeof(MT) == 4)
      bsr3_row_widen<G>(rowptr, colidx, vals, x, r, gl, mask, y0, y1, y2);
    else
      bsr3_row<G, MT, double, double>(rowptr, colidx, vals, x, r, gl, mask, y0, y1, y2);
    // lanes 0..2 (all hold the sums) take a component each
    if (gl < 3) {
      const double rv = b[r * 3 + gl] - (gl == 0 ? y0 : (gl == 1 ? y1 : y2));
      rhi[r * 3 + gl] = rv;
      acc = fma(rv, rv, acc);
    }
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// r_hi = b - A x for an FP32 3x3 matrix without FP64 multiply-adds, which
// are scarce on this GPU.  x arrives split into floats xh + xl (48
// significant bits); each product a*xh is split exactly by the FMA residual
// and summed with TwoSum into a float pair per row component, a*xl goes into
// the low part (the compensated dot product of Ogita, Rump and Oishi, 2005);
// the lanes of a row combine their pairs the same way and lane 0 converts
// once to FP64 for b - y.  The error is about 2^-46 of sum |a||x| against
// 2^-52 for FP64 accumulation: ample for the residual replacement between
// checks, whose residual is never below the tolerance.  A residual that
// meets the tolerance is recomputed with k_true_residual3 before the solver
// accepts it.
template <int G>
__global__ void __launch_bounds__(RED_T)
    k_true_residual3c(int32_t n, const uint32_t *__restrict__ rowptr,
                      const uint32_t *__restrict__ colidx, const float *__restrict__ vals,
                      const float *__restrict__ xh, const float *__restrict__ xl,
                      const double *__restrict__ b, double *__restrict__ rhi,
                      double *__restrict__ part) {
  __shared__ double sh[33];
  const int gl = threadIdx.x & (G - 1);
  const unsigned mask = group_mask<G>();
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x / G);
  double acc = 0;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; r < n; r += stride) {
    float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
    const uint32_t e = rowptr[r + 1];
    for (uint32_t q = rowptr[r] + gl; q < e; q += G) {
      const uint32_t c = colidx[q];
      const float *v = vals + (size_t)q * 9;
      float xa[3], xb[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        xa[k] = ldg(xh + (size_t)c * 3 + k);
        xb[k] = ldg(xl + (size_t)c * 3 + k);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float a = ldg(v + i * 3 + k);
          const float p = __fmul_rn(a, xa[k]);
          const float pe = __fmaf_rn(a, xa[k], -p);  // a*xh - p, exact
          float s, se;
          two_sum(h[i], p, s, se);
          h[i] = s;
          l[i] = __fadd_rn(l[i], __fadd_rn(se, __fmaf_rn(a, xb[k], pe)));
        }
    }
#pragma unroll
    for (int o = G >> 1; o > 0; o >>= 1)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float oh = __shfl_xor_sync(mask, h[i], o, G);
        const float ol = __shfl_xor_sync(mask, l[i], o, G);
        float s, se;
        two_sum(h[i], oh, s, se);
        h[i] = s;
        l[i] = __fadd_rn(__fadd_rn(l[i], ol), se);
      }
    // every lane holds the row's sums: lanes 0..2 take a component each,
    // so the FP64 pipe (a small fraction of the FP32 rate on this GPU) sees
    // one add, one subtract and one multiply-add per component, the
    // conversions done by integer operations
    if (gl < 3) {
      const float hv = gl == 0 ? h[0] : (gl == 1 ? h[1] : h[2]);
      const float lv = gl == 0 ? l[0] : (gl == 1 ? l[1] : l[2]);
      const double y = widen_f32(hv) + widen_f32(lv);
      const double rv = b[r * 3 + gl] - y;
      rhi[r * 3 + gl] = rv;
      acc = fma(rv, rv, acc);
    }
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// x_hi += x_lo, x_lo = 0, and the float split xh + xl of the new x_hi.
template <typename XT>
__global__ void k_fold_split(int64_t len, double *__restrict__ xhi, XT *__restrict__ xlo,
                             float *__restrict__ xh, float *__restrict__ xl) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = xhi[i] + (double)xlo[i];
    xhi[i] = x;
    xlo[i] = XT(0);
    const float a = (float)x;
    xh[i] = a;
    xl[i] = (float)(x - (double)a);
  }
}

// The float split xh + xl of x.
static __global__ void __launch_bounds__(RED_T) k_split_x(int64_t len, const double *__restrict__ x,
                                                   float *__restrict__ xh,
                                                   float *__restrict__ xl) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float a = (float)x[i];
    xh[i] = a;
    xl[i] = (float)(x[i] - (double)a);
  }
}

// Any bs (one thread per row).
template <typename MT>
__global__ void k_true_residual_any(int32_t n, int32_t bs, const uint32_t *__restrict__ rowptr,
                                    const uint32_t *__restrict__ colidx,
                                    const MT *__restrict__ vals, const double *__restrict__ x,
                                    const double *__restrict__ b, double *__restrict__ rhi,
                                    double *__restrict__ part) {
  __shared__ double sh[33];
  double acc = 0;
  for (int64_t qq = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; qq < n;
       qq += (int64_t)gridDim.x * blockDim.x) {
    for (int q1 = 0; q1 < bs; ++q1) {
      double s = 0;
      for (uint32_t qp = rowptr[qq]; qp < rowptr[qq + 1]; ++qp) {
        const int64_t c = colidx[qp];
        double t = 0;
        for (int p1 = 0; p1 < bs; ++p1)
          t += (double)vals[(size_t)qp * bs * bs + q1 * bs + p1] * x[c * bs + p1];
        s += t;
      }
      const double rv = b[qq * bs + q1] - s;
      rhi[qq * bs + q1] = rv;
      acc += rv * rv;
    }
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Point-Jacobi inverse diagonal (VT) from the diagonal blocks; bs3 = 1 also
// writes the inverted 3x3 diagonal blocks (block Jacobi).  PACK6: the block
// inverse symmetrised ((M + M^T) / 2 in FP64) and stored as its upper
// triangle m00 m01 m02 m11 m12 m22, 6 values per vertex (the mixed solver's
// layout: a third fewer bytes per K2, and an exactly symmetric M).
template <typename MT, typename VT, bool PACK6 = false>
__global__ void k_diag_inv(int32_t n, int32_t bs, const uint32_t *__restrict__ rowptr,
                           const uint32_t *__restrict__ colidx, const MT *__restrict__ vals,
                           VT *__restrict__ dinv, int block3, int *err) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = rowptr[v], hi = rowptr[v + 1];
    const uint32_t end = hi;
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (colidx[mid] < (uint32_t)v) lo = mid + 1; else hi = mid;
    }
    const int per = block3 ? (PACK6 ? 6 : 9) : bs;
    if (lo >= end || colidx[lo] != (uint32_t)v) {
      atomicCAS(err, 0, 5 /* DEV_NO_DIAGONAL */);
      for (int k = 0; k < per; ++k) dinv[v * per + k] = VT(0);
      continue;
    }
    const MT *D = vals + (size_t)lo * bs * bs;
    if (!block3) {
      for (int k = 0; k < bs; ++k) {
        const double d = (double)D[k * bs + k];
        dinv[v * bs + k] = d != 0.0 ? (VT)(1.0 / d) : VT(0);
      }
    } else {
      double a[9];
      for (int k = 0; k < 9; ++k) a[k] = (double)D[k];
      const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8],
                   c02 = a[3] * a[7] - a[4] * a[6];
      const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
      if (det == 0.0 || !isfinite(det)) {  // singular block: fall back to point Jacobi
        for (int k = 0; k < per; ++k) dinv[v * per + k] = VT(0);
        for (int k = 0; k < 3; ++k)
          dinv[v * per + (PACK6 ? (k == 0 ? 0 : (k == 1 ? 3 : 5)) : k * 4)] =
              a[k * 4] != 0.0 ? (VT)(1.0 / a[k * 4]) : VT(0);
        continue;
      }
      const double id = 1.0 / det;
      const double inv[9] = {c00 * id, (a[2] * a[7] - a[1] * a[8]) * id, (a[1] * a[5] - a[2] * a[4]) * id,
                             c01 * id, (a[0] * a[8] - a[2] * a[6]) * id, (a[2] * a[3] - a[0] * a[5]) * id,
                             c02 * id, (a[1] * a[6] - a[0] * a[7]) * id, (a[0] * a[4] - a[1] * a[3]) * id};
      if (PACK6) {
        VT *m = dinv + v * 6;
        m[0] = (VT)inv[0];
        m[1] = (VT)(0.5 * (inv[1] + inv[3]));
        m[2] = (VT)(0.5 * (inv[2] + inv[6]));
        m[3] = (VT)inv[4];
        m[4] = (VT)(0.5 * (inv[5] + inv[7]));
        m[5] = (VT)inv[8];
      } else {
        for (int k = 0; k < 9; ++k) dinv[v * 9 + k] = (VT)inv[k];
      }
    }
  }
}

}  // namespace sg
