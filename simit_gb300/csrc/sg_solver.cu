// CG / PCG solver runtime: workspace, graph-captured iteration batches and the
// host decisions taken only at rare check points (true residual, reliable
// update, convergence).
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "sg_internal.cuh"
#include "sg_solver_kernels.cuh"
#include "sg_solver.h"
#include "sg_spmv_api.h"

namespace sg {

__global__ void k_sum_parts(const double *part, int np, double *out) {
  __shared__ double sh[33];
  double t = sum_parts(part, np, sh);
  if (threadIdx.x == 0) *out = t;
}

template <typename VT>
__global__ void k_cast_r(int64_t len, const double *__restrict__ rhi, VT *__restrict__ r) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    r[i] = (VT)rhi[i];
}

// x += a p: the last iteration's update when K2 stopped the batch and K3,
// which applies it otherwise, returned early.
__global__ void k_x_pending(int64_t len, float a, const float *__restrict__ p,
                            float *__restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = x[i] + a * p[i];
}

template <typename XT>
__global__ void k_add_lo(int64_t len, double *__restrict__ xhi, XT *__restrict__ xlo) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    xhi[i] += (double)xlo[i];
    xlo[i] = XT(0);
  }
}

// z = M r (M from dinv), partial sums of r.z.
template <typename VT, int PREC>
__global__ void __launch_bounds__(RED_T) k_prec_dot(int64_t len, const VT *__restrict__ r,
                                                    const VT *__restrict__ dinv,
                                                    VT *__restrict__ z, double *__restrict__ part) {
  __shared__ double sh[33];
  double acc = 0;
  if (PREC == PK_BLOCK3) {
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v * 3 < len;
         v += (int64_t)gridDim.x * blockDim.x) {
      const VT r0 = r[v * 3], r1 = r[v * 3 + 1], r2 = r[v * 3 + 2];
      VT zz[3];
      if (sizeof(VT) == 4) {  // mixed: packed symmetric inverse (k_diag_inv PACK6)
        const VT *m = dinv + v * 6;
        zz[0] = m[0] * r0 + m[1] * r1 + m[2] * r2;
        zz[1] = m[1] * r0 + m[3] * r1 + m[4] * r2;
        zz[2] = m[2] * r0 + m[4] * r1 + m[5] * r2;
      } else {
        const VT *D = dinv + v * 9;
#pragma unroll
        for (int k = 0; k < 3; ++k) zz[k] = D[k * 3] * r0 + D[k * 3 + 1] * r1 + D[k * 3 + 2] * r2;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        z[v * 3 + k] = zz[k];
        acc += (double)r[v * 3 + k] * (double)zz[k];
      }
    }
  } else {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
      VT zi = r[i];
      if (PREC == PK_JACOBI) zi = dinv[i] * zi;
      if (PREC != PK_NONE) z[i] = zi;
      acc += (double)r[i] * (double)zi;
    }
  }
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

template <typename VT>
__global__ void k_p_update(int64_t len, const VT *__restrict__ z, double beta, VT *__restrict__ p) {
  const VT b = (VT)beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + b * p[i];
}

__global__ void __launch_bounds__(RED_T) k_dot2(int64_t len, const double *__restrict__ a,
                                               const double *__restrict__ b,
                                               double *__restrict__ part) {
  __shared__ double sh[33];
  double acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    acc += a[i] * b[i];
  double t = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_f64_to_f32(int64_t len, const double *__restrict__ a, float *__restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

__global__ void k_f32_to_f64(int64_t len, const float *__restrict__ a, double *__restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

// ---------------------------------------------------------------------------
enum Kind { KIND_F64 = 0, KIND_F64_M32 = 1, KIND_MIXED = 2 };

static int alloc_dev(Solver *S, void **p, size_t bytes) {
  if (bytes == 0) bytes = 256;
  SG_CHECK_CUDA(cudaMalloc(p, bytes));
  S->allocs.push_back(*p);
  return SG_OK;
}

template <typename MT, typename VT>
static int launch_k1(Solver *S, cudaStream_t st) {
  const sg_matrix &A = S->A;
  if (S->sym)
    return sym_launch(S->sym, st, S->ctl, true, (const float *)S->p, (float *)S->q, S->part1);
  if (S->tma) {
    const int vdt = sizeof(MT) == 8 ? SG_F64 : SG_F32, xdt = sizeof(VT) == 8 ? SG_F64 : SG_F32;
    return bsr3_tma_launch(S->c, st, S->ctl, A.bs, vdt, xdt, S->tma_var, 1, A.n, A.rowptr,
                           A.colidx, S->bulk_vals, S->p, S->q, S->part1, S->pstats, S->P1,
                           S->tma_smem);
  }
  const MT *vals = (const MT *)S->bulk_vals;
  const VT *p = (const VT *)S->p;
  VT *q = (VT *)S->q;
#define SG_K1(BSV, GV)                                                                       \
  k_cg_spmv<BSV, GV, MT, VT><<<S->P1, RED_T, 0, st>>>(S->ctl, A.n, A.bs, A.rowptr, A.colidx, \
                                                      vals, p, q, S->part1)
  if (A.bs == 3 || A.bs == 1) {
    switch (S->G) {
      case 1: if (A.bs == 3) SG_K1(3, 1); else SG_K1(1, 1); break;
      case 2: if (A.bs == 3) SG_K1(3, 2); else SG_K1(1, 2); break;
      case 4: if (A.bs == 3) SG_K1(3, 4); else SG_K1(1, 4); break;
      case 8: if (A.bs == 3) SG_K1(3, 8); else SG_K1(1, 8); break;
      case 16: if (A.bs == 3) SG_K1(3, 16); else SG_K1(1, 16); break;
      default: if (A.bs == 3) SG_K1(3, 32); else SG_K1(1, 32); break;
    }
  } else {
    SG_K1(0, 1);
  }
#undef SG_K1
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <int PREC>
static void launch_k2_v4(Solver *S, cudaStream_t st, int par) {
  k_cg_update_v4<PREC, PREC != PK_EXTERNAL><<<S->P2, RED_T, 0, st>>>(
      S->ctl, par, S->len, S->part1, S->P1, S->tma, (const float *)S->p, (const float *)S->q,
      (float *)S->r, (float *)S->xupd, (float *)S->z, (const float *)S->dinv, S->part2);
}

template <typename VT, typename XT>
static int launch_k2(Solver *S, cudaStream_t st, int par) {
  if (S->ext_k2) return S->ext_k2(S, st, par);
  const VT *p = (const VT *)S->p, *q = (const VT *)S->q, *dinv = (const VT *)S->dinv;
  VT *r = (VT *)S->r, *z = (VT *)S->z;
  XT *x = (XT *)S->xupd;
  if (sizeof(VT) == 4 && sizeof(XT) == 4) {
    switch (S->prec) {
      case PK_NONE: launch_k2_v4<PK_NONE>(S, st, par); break;
      case PK_JACOBI: launch_k2_v4<PK_JACOBI>(S, st, par); break;
      case PK_BLOCK3: {
        static PerDeviceOnce attr;
        const size_t sm = K2W_WARPS * sizeof(K2WarpSmem);
        SG_TRY(once_per_device(attr, S->c->device, [&]() -> int {
          SG_CHECK_CUDA(cudaFuncSetAttribute(k_cg_update_w<true, false>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
          return SG_OK;
        }));
        const int64_t nchunks = (S->len / 12 + 31) / 32;
        int64_t grid = (nchunks + K2W_WARPS - 1) / K2W_WARPS;
        // 2 CTAs of 8 warps per SM (3 fit, and measured 3 % slower per step)
        if (grid > 2 * (int64_t)S->c->num_sms) grid = 2 * (int64_t)S->c->num_sms;
        if (grid < 1) grid = 1;
        S->k3_xupd = 1;  // x += alpha p moves to K3
        SG_CHECK_CUDA(launch_k(S->c, k_cg_update_w<true, false>, (int)grid, K2W_WARPS * 32, sm, st,
                               S->ctl, par, S->len, (const double *)S->part1, S->P1, S->tma,
                               (const float *)S->p, (const float *)S->q, (float *)S->r,
                               (float *)S->xupd, (float *)S->z, (const float *)S->dinv,
                               S->part2));
        break;
      }
      default: launch_k2_v4<PK_EXTERNAL>(S, st, par); break;
    }
    SG_CHECK_LAUNCH();
    return SG_OK;
  }
  switch (S->prec) {
    case PK_NONE:
      k_cg_update<VT, XT, PK_NONE><<<S->P2, RED_T, 0, st>>>(S->ctl, par, S->len, S->part1, S->P1,
                                                            p, q, r, x, z, dinv, S->part2);
      break;
    case PK_JACOBI:
      k_cg_update<VT, XT, PK_JACOBI><<<S->P2, RED_T, 0, st>>>(S->ctl, par, S->len, S->part1,
                                                              S->P1, p, q, r, x, z, dinv, S->part2);
      break;
    case PK_BLOCK3:
      k_cg_update<VT, XT, PK_BLOCK3><<<S->P2, RED_T, 0, st>>>(S->ctl, par, S->len, S->part1,
                                                              S->P1, p, q, r, x, z, dinv, S->part2);
      break;
    default:
      k_cg_update<VT, XT, PK_EXTERNAL><<<S->P2, RED_T, 0, st>>>(
          S->ctl, par, S->len, S->part1, S->P1, p, q, r, x, z, dinv, S->part2);
      break;
  }
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <typename VT>
static int launch_k3(Solver *S, cudaStream_t st, int par) {
  const VT *z = (const VT *)(S->prec == PK_NONE ? S->r : S->z);
  const int np2 = S->np2_ext > 0 ? S->np2_ext : S->P2;
  // K2 decided, unless an external preconditioner ran after it and did not
  if (sizeof(VT) == 4)
    SG_CHECK_CUDA(launch_k(S->c, k_cg_direction_v4, S->P2, RED_T, 0, st, S->ctl, par, S->len,
                           (const double *)S->part2, np2,
                           (int)(S->prec != PK_EXTERNAL || S->ext_decides),
                           (const float *)z, (float *)S->p, (float *)S->xupd, S->k3_xupd));
  else
    k_cg_direction<VT><<<S->P2, RED_T, 0, st>>>(S->ctl, par, S->len, S->part2, S->P2, z,
                                                (VT *)S->p);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <typename MT, typename VT, typename XT>
static int capture_batch(Solver *S) {
  cudaStream_t st = S->c->stream;
  cudaGraph_t g = nullptr;
  SG_CHECK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int rc = SG_OK;
  // optional programmatic dependent launch for the kernels launched through
  // launch_k (K1 per-warp TMA SpMV, K2 warp-staged update, K3 FP32 direction)
  S->c->pdl = S->o.pdl != 0;
  for (int k = 0; k < S->batch && rc == SG_OK; ++k) {
    const int par = k & 1;
    rc = launch_k1<MT, VT>(S, st);
    if (rc == SG_OK) rc = launch_k2<VT, XT>(S, st, par);
    if (rc == SG_OK && S->ext_prec) rc = S->ext_prec(S, st, par);
    if (rc == SG_OK) rc = launch_k3<VT>(S, st, par);
  }
  S->c->pdl = false;
  cudaError_t e = cudaStreamEndCapture(st, &g);
  if (rc != SG_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  SG_CHECK_CUDA(e);
  SG_CHECK_CUDA(cudaGraphInstantiate(&S->gexec, g, 0));
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  S->graph_kernels = (int64_t)nn;
  cudaGraphDestroy(g);
  return SG_OK;
}

// r_hi = b - A x_hi in FP64 (FP64 accumulation); returns ||r_hi||^2 (sync).
static int true_residual(Solver *S, const double *b, double *rr) {
  const sg_matrix &A = S->A;
  S->launches += 2;
  cudaStream_t st = S->c->stream;
  const int PT = S->P1;
  if (A.bs == 3) {
    if (A.dtype == SG_F64)
      k_true_residual3<4, double><<<PT, RED_T, 0, st>>>(A.n, A.rowptr, A.colidx,
                                                         (const double *)A.vals, S->xw, b,
                                                         S->rhi, S->part3);
    else
      k_true_residual3<4, float><<<PT, RED_T, 0, st>>>(A.n, A.rowptr, A.colidx,
                                                        (const float *)A.vals, S->xw, b, S->rhi,
                                                        S->part3);
  } else {
    if (A.dtype == SG_F64)
      k_true_residual_any<double><<<PT, RED_T, 0, st>>>(A.n, A.bs, A.rowptr, A.colidx,
                                                         (const double *)A.vals, S->xw, b,
                                                         S->rhi, S->part3);
    else
      k_true_residual_any<float><<<PT, RED_T, 0, st>>>(A.n, A.bs, A.rowptr, A.colidx,
                                                        (const float *)A.vals, S->xw, b, S->rhi,
                                                        S->part3);
  }
  SG_CHECK_LAUNCH();
  k_sum_parts<<<1, RED_T, 0, st>>>(S->part3, PT, S->dres);
  SG_CHECK_LAUNCH();
  SG_CHECK_CUDA(cudaMemcpyAsync(S->c->h_stage, S->dres, 8, cudaMemcpyDeviceToHost, st));
  SG_CHECK_CUDA(cudaStreamSynchronize(st));
  *rr = *(double *)S->c->h_stage;
  return SG_OK;
}

// The same residual from the float split of x_hi without FP64 multiply-adds
// (k_true_residual3c); S->xsplit must hold the split of the current x_hi.
static int true_residual_fast(Solver *S, const double *b, double *rr) {
  const sg_matrix &A = S->A;
  S->launches += 2;
  cudaStream_t st = S->c->stream;
  const int PT = S->P1;
  k_true_residual3c<4><<<PT, RED_T, 0, st>>>(A.n, A.rowptr, A.colidx, (const float *)A.vals,
                                             S->xsplit, S->xsplit + S->len, b, S->rhi,
                                             S->part3);
  SG_CHECK_LAUNCH();
  k_sum_parts<<<1, RED_T, 0, st>>>(S->part3, PT, S->dres);
  SG_CHECK_LAUNCH();
  SG_CHECK_CUDA(cudaMemcpyAsync(S->c->h_stage, S->dres, 8, cudaMemcpyDeviceToHost, st));
  SG_CHECK_CUDA(cudaStreamSynchronize(st));
  *rr = *(double *)S->c->h_stage;
  return SG_OK;
}

// r = (VT) r_hi; z = M r (or the external preconditioner); returns r.z (sync).
template <typename VT>
static int restart_from_rhi(Solver *S, double *rz) {
  cudaStream_t st = S->c->stream;
  S->launches += 3;
  k_cast_r<VT><<<S->P2, RED_T, 0, st>>>(S->len, S->rhi, (VT *)S->r);
  SG_CHECK_LAUNCH();
  if (S->ext_prec_apply) {
    SG_TRY(S->ext_prec_apply(S, st));
  } else {
    switch (S->prec) {
      case PK_NONE:
        k_prec_dot<VT, PK_NONE><<<S->P2, RED_T, 0, st>>>(S->len, (VT *)S->r, (VT *)S->dinv,
                                                         (VT *)S->z, S->part3);
        break;
      case PK_JACOBI:
        k_prec_dot<VT, PK_JACOBI><<<S->P2, RED_T, 0, st>>>(S->len, (VT *)S->r, (VT *)S->dinv,
                                                           (VT *)S->z, S->part3);
        break;
      default:
        k_prec_dot<VT, PK_BLOCK3><<<S->P2, RED_T, 0, st>>>(S->len, (VT *)S->r, (VT *)S->dinv,
                                                           (VT *)S->z, S->part3);
        break;
    }
    SG_CHECK_LAUNCH();
  }
  k_sum_parts<<<1, RED_T, 0, st>>>(S->part3, S->P2, S->dres);
  SG_CHECK_LAUNCH();
  SG_CHECK_CUDA(cudaMemcpyAsync(S->c->h_stage, S->dres, 8, cudaMemcpyDeviceToHost, st));
  SG_CHECK_CUDA(cudaStreamSynchronize(st));
  *rz = *(double *)S->c->h_stage;
  return SG_OK;
}

template <typename MT, typename VT, typename XT>
static int solve_impl(Solver *S, const double *b, double *x, sg_solve_result *res) {
  Ctx *c = S->c;
  cudaStream_t st = c->stream;
  const bool mixed = S->kind == KIND_MIXED;
  memset(res, 0, sizeof(*res));
  S->launches = 0;
  if (S->x_zero)
    SG_CHECK_CUDA(cudaMemsetAsync(S->xw, 0, S->len * 8, st));
  else
    SG_CHECK_CUDA(cudaMemcpyAsync(S->xw, x, S->len * 8, cudaMemcpyDeviceToDevice, st));
  SG_CHECK_CUDA(cudaMemsetAsync(S->ctl, 0, sizeof(SolveCtl), st));
  if (mixed) SG_CHECK_CUDA(cudaMemsetAsync(S->xlo, 0, S->len * sizeof(XT), st));
  // b'b
  dot_launch(c, S->len, b, b, S->part3, S->dres);
  S->launches += 2;
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, S->dres, 8, cudaMemcpyDeviceToHost, st));
  SG_CHECK_CUDA(cudaStreamSynchronize(st));
  const double bb = *(double *)c->h_stage;
  res->bnorm2 = bb;
  double tol2;
  switch (S->o.stop) {
    case SG_STOP_NORMR2: tol2 = S->o.tol; break;
    case SG_STOP_NORMR: tol2 = S->o.tol * S->o.tol; break;
    default: tol2 = S->o.tol * S->o.tol * bb; break;
  }
  // Checks run the compensated FP32 residual when the matrix is FP32; one
  // that meets the tolerance (with 10 % slack in the norm) is recomputed with
  // FP64 accumulation, and only that decides convergence.
  const bool fast = S->xsplit != nullptr;
  bool exact = false;  // the last residual was the FP64 one
  auto check = [&](double *out) -> int {
    if (fast) {
      k_fold_split<XT><<<S->P2, RED_T, 0, st>>>(S->len, S->xw, (XT *)S->xlo, S->xsplit,
                                                 S->xsplit + S->len);
      SG_CHECK_LAUNCH();
      S->launches += 1;
      SG_TRY(true_residual_fast(S, b, out));
      if (std::isfinite(*out) && *out > 1.21 * tol2) {
        exact = false;
        return SG_OK;
      }
    } else if (mixed) {
      k_add_lo<XT><<<S->P2, RED_T, 0, st>>>(S->len, S->xw, (XT *)S->xlo);
      SG_CHECK_LAUNCH();
      S->launches += 1;
    }
    exact = true;
    return true_residual(S, b, out);
  };
  double rr = 0;
  if (S->x_zero) {
    // x = 0: the residual is b itself, exactly (no SpMV, no split of x)
    SG_CHECK_CUDA(cudaMemcpyAsync(S->rhi, b, S->len * 8, cudaMemcpyDeviceToDevice, st));
    rr = bb;
    exact = true;
  } else {
    SG_TRY(check(&rr));
  }
  res->normr2 = rr;
  res->true_normr2 = rr;
  int iters = 0;
  int status = 0;
  if (!(rr > tol2)) status = SG_STATUS_CONVERGED;
  if (!std::isfinite(rr)) status = SG_STATUS_NAN;
  double rz = 0;
  int fallback = 0;
  if (!status) SG_TRY(restart_from_rhi<VT>(S, &rz));
  if (!status && S->flexible && !(rz > 0.0)) {
    // the variable preconditioner gives no descent direction from the start:
    // switch to its fallback (block Jacobi) before the first iteration
    fallback = 1;
    res->fallbacks++;
    const int one = 1;
    SG_CHECK_CUDA(cudaMemcpyAsync((char *)S->ctl + offsetof(SolveCtl, fallback), &one,
                                  sizeof(int), cudaMemcpyHostToDevice, st));
    SG_TRY(restart_from_rhi<VT>(S, &rz));
  }
  if (!status) {
    const VT *z = (const VT *)(S->prec == PK_NONE ? S->r : S->z);
    SG_CHECK_CUDA(cudaMemcpyAsync(S->p, z, S->len * sizeof(VT), cudaMemcpyDeviceToDevice, st));
  }
  const double delta = S->o.reliable_delta > 0 ? S->o.reliable_delta : 0.1;
  double rr_ref = rr;
  SolveCtl *h = S->hctl;
  while (!status) {
    // (re)start a batch with the current state in parity slot 0
    memset(h, 0, sizeof(*h));
    h->status = ST_RUNNING;
    h->iter[0] = h->iter[1] = iters;
    h->maxiters = S->o.maxiters;
    h->check_every = S->o.check_every;
    h->flexible = S->flexible;
    h->rz[0] = h->rz[1] = rz;
    h->tol2 = tol2;
    h->upd2 = mixed ? delta * delta * rr_ref : 0.0;
    h->fallback = fallback;
    if (iters >= S->o.maxiters) {
      status = SG_STATUS_MAXITER;
      break;
    }
    SG_CHECK_CUDA(cudaMemcpyAsync(S->ctl, h, sizeof(SolveCtl), cudaMemcpyHostToDevice, st));
    for (;;) {
      SG_CHECK_CUDA(cudaGraphLaunch(S->gexec, st));
      S->launches += S->graph_kernels;
      SG_CHECK_CUDA(cudaMemcpyAsync(h, S->ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, st));
      SG_CHECK_CUDA(cudaStreamSynchronize(st));
      if (h->status != ST_RUNNING) break;
      // a variable preconditioner that lets the residual grow 100x over the
      // last reference point is abandoned for block Jacobi
      if (S->flexible && !h->fallback && h->last_rr > 1e4 * rr_ref) {
        SolveCtl one = *h;
        one.fallback = 1;
        one.status = ST_NEED_CHECK;
        SG_CHECK_CUDA(cudaMemcpyAsync(S->ctl, &one, sizeof(SolveCtl), cudaMemcpyHostToDevice, st));
        SG_CHECK_CUDA(cudaStreamSynchronize(st));
        *h = one;
        break;
      }
    }
    exact = false;  // x moved since the last residual
    if (S->k3_xupd && (h->status == ST_NEED_CHECK || h->status == ST_MAXITER)) {
      // K2 updated r with alpha and stopped the batch; K3 returned early
      k_x_pending<<<S->P2, RED_T, 0, st>>>(S->len, (float)h->last_alpha, (const float *)S->p,
                                           (float *)S->xupd);
      SG_CHECK_LAUNCH();
      S->launches += 1;
    }
    // the slot K3 wrote last holds the larger iteration count
    const int cur = h->iter[1] > h->iter[0] ? 1 : 0;
    iters = h->iter[cur];
    res->normr2 = h->last_rr;
    if (h->status == ST_BREAKDOWN) status = SG_STATUS_BREAKDOWN;
    else if (h->status == ST_NAN) status = SG_STATUS_NAN;
    if (status) break;
    // ST_NEED_CHECK or ST_MAXITER: fold x_lo in, look at the true residual
    const bool iter_conv = h->last_rr <= tol2;
    if (!S->o.verify && !mixed && iter_conv) {
      status = SG_STATUS_CONVERGED;
      break;
    }
    res->checks++;
    SG_TRY(check(&rr));
    if (!std::isfinite(rr)) {
      status = SG_STATUS_NAN;
      break;
    }
    if (rr <= tol2 && (S->o.verify || iter_conv || mixed)) {
      status = SG_STATUS_CONVERGED;
      break;
    }
    if (h->status == ST_MAXITER || iters >= S->o.maxiters) {
      status = SG_STATUS_MAXITER;
      break;
    }
    // residual replacement: continue from the true residual, same direction
    // (a fresh direction after a switch to the fallback preconditioner)
    const bool switched = h->fallback && !fallback;
    if (switched) {
      fallback = 1;
      res->fallbacks++;
    }
    const double rz_old = h->rz[cur ^ 1];
    double rz_new = 0;
    SG_TRY(restart_from_rhi<VT>(S, &rz_new));
    const VT *z = (const VT *)(S->prec == PK_NONE ? S->r : S->z);
    k_p_update<VT><<<S->P2, RED_T, 0, st>>>(S->len, z, switched ? 0.0 : rz_new / rz_old,
                                            (VT *)S->p);
    S->launches += 1;
    SG_CHECK_LAUNCH();
    rz = rz_new;
    rr_ref = rr;
  }
  if (mixed && status) {
    k_add_lo<XT><<<S->P2, RED_T, 0, st>>>(S->len, S->xw, (XT *)S->xlo);
    SG_CHECK_LAUNCH();
    S->launches += 1;
  }
  SG_CHECK_CUDA(cudaMemcpyAsync(x, S->xw, S->len * 8, cudaMemcpyDeviceToDevice, st));
  if (status == SG_STATUS_CONVERGED && exact) {
    // converged on an FP64 residual of this very x (x_lo was folded into
    // x_hi before it, so the fold above added zeros)
    res->true_normr2 = rr;
  } else if (S->o.verify || mixed) {
    double rt = 0;
    SG_TRY(true_residual(S, b, &rt));
    res->true_normr2 = rt;
  } else {
    res->true_normr2 = rr;
  }
  SG_CHECK_CUDA(cudaStreamSynchronize(st));
  res->status = status;
  res->iters = iters;
  res->kernels = S->launches;
  return SG_OK;
}

}  // namespace sg

using namespace sg;

extern "C" {

int sg_solver_create(sg_ctx *h, const sg_matrix *A, const sg_solve_opts *o, sg_solver **out) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && A && o && out, "sg_solver_create: null argument");
  SG_REQUIRE(A->n >= 1 && A->bs >= 1 && A->rowptr && A->colidx && A->vals,
             "sg_solver_create: bad matrix");
  SG_REQUIRE(A->dtype == SG_F32 || A->dtype == SG_F64, "sg_solver_create: dtype");
  SG_REQUIRE(o->precision == SG_SOLVE_F64 || o->precision == SG_SOLVE_MIXED,
             "sg_solver_create: precision %d", o->precision);
  SG_REQUIRE(o->precond >= SG_PRECOND_NONE && o->precond <= SG_PRECOND_LEARNED,
             "sg_solver_create: precond %d", o->precond);
  SG_REQUIRE(o->precond != SG_PRECOND_LEARNED ||
                 (o->learned_params && A->bs == 3 && o->precision == SG_SOLVE_MIXED),
             "sg_solver_create: the learned preconditioner needs learned_params, bs = 3 and "
             "SG_SOLVE_MIXED");
  SG_REQUIRE(o->precond != SG_PRECOND_BLOCK_JACOBI || A->bs == 3,
             "sg_solver_create: block Jacobi needs bs = 3");
  SG_REQUIRE(o->maxiters >= 0, "sg_solver_create: maxiters");
  SG_REQUIRE(o->storage == SG_STORAGE_FULL || o->storage == SG_STORAGE_SYMMETRIC,
             "sg_solver_create: storage %d", o->storage);
  Solver *S = new Solver();
  int rc = o->precond == SG_PRECOND_LEARNED
               ? learned_solver_init(c, A, o, o->learned_params, S)
               : solver_init(c, A, o, S, nullptr);
  if (rc != SG_OK) {
    solver_free(S);
    return rc;
  }
  *out = reinterpret_cast<sg_solver *>(S);
  return SG_OK;
}

int sg_solver_solve(sg_solver *hs, const double *b, double *x, sg_solve_result *res) {
  Solver *S = reinterpret_cast<Solver *>(hs);
  DeviceGuard dg_(S ? S->c : nullptr);
  SG_REQUIRE(S && b && x && res, "sg_solver_solve: null argument");
  return solver_solve(S, b, x, res);
}

int sg_solver_solve_ex(sg_solver *hs, const void *b, int b_dtype, double *x, int x_zero,
                       sg_solve_result *res) {
  Solver *S = reinterpret_cast<Solver *>(hs);
  DeviceGuard dg_(S ? S->c : nullptr);
  SG_REQUIRE(S && b && x && res, "sg_solver_solve_ex: null argument");
  SG_REQUIRE(b_dtype == SG_F32 || b_dtype == SG_F64, "sg_solver_solve_ex: b_dtype %d", b_dtype);
  const double *b64 = (const double *)b;
  if (b_dtype == SG_F32) {
    if (!S->b64) {
      SG_CHECK_CUDA(cudaMalloc((void **)&S->b64, (size_t)S->len * 8 + 8));
      S->allocs.push_back(S->b64);
    }
    k_f32_to_f64<<<S->P2, RED_T, 0, S->c->stream>>>(S->len, (const float *)b, S->b64);
    SG_CHECK_LAUNCH();
    b64 = S->b64;
  }
  S->x_zero = x_zero ? 1 : 0;
  const int rc = solver_solve(S, b64, x, res);
  S->x_zero = 0;
  if (rc == SG_OK && b_dtype == SG_F32) res->kernels += 1;
  return rc;
}

int sg_solver_refresh(sg_solver *hs) {
  Solver *S = reinterpret_cast<Solver *>(hs);
  DeviceGuard dg_(S ? S->c : nullptr);
  SG_REQUIRE(S, "sg_solver_refresh: null solver");
  return refresh_matrix(S);
}

int sg_solver_destroy(sg_solver *hs) {
  Solver *S = reinterpret_cast<Solver *>(hs);
  DeviceGuard dg_(S ? S->c : nullptr);
  solver_free(S);
  return SG_OK;
}

int sg_residual(sg_ctx *h, const sg_matrix *A, const double *x, const double *b, double *r,
                double *h_rr, int mode) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && A && x && b && r && h_rr, "sg_residual: null argument");
  SG_REQUIRE(A->n >= 1 && A->bs >= 1 && A->rowptr && A->colidx && A->vals,
             "sg_residual: bad matrix");
  SG_REQUIRE(A->dtype == SG_F32 || A->dtype == SG_F64, "sg_residual: dtype");
  SG_REQUIRE(mode == SG_RESIDUAL_FP64 ||
                 (mode == SG_RESIDUAL_COMPENSATED && A->dtype == SG_F32 && A->bs == 3),
             "sg_residual: mode %d (compensated needs an FP32 3x3 matrix)", mode);
  cudaStream_t st = c->stream;
  const int64_t len = (int64_t)A->n * A->bs;
  const int PT = grid_for(c, (int64_t)A->n * 4, RED_T, 8);
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(PT, 8) + Scratch::bytes_for(1, 8) +
                   (mode ? Scratch::bytes_for(len * 2, 4) : 0) + 1024));
  double *part = s.alloc<double>(PT), *dres = s.alloc<double>(1);
  if (mode == SG_RESIDUAL_COMPENSATED) {
    float *xs = s.alloc<float>(len * 2);
    k_split_x<<<grid_for(c, len, RED_T, 8), RED_T, 0, st>>>(len, x, xs, xs + len);
    SG_CHECK_LAUNCH();
    k_true_residual3c<4><<<PT, RED_T, 0, st>>>(A->n, A->rowptr, A->colidx,
                                               (const float *)A->vals, xs, xs + len, b, r, part);
  } else if (A->bs == 3) {
    if (A->dtype == SG_F64)
      k_true_residual3<4, double><<<PT, RED_T, 0, st>>>(A->n, A->rowptr, A->colidx,
                                                         (const double *)A->vals, x, b, r, part);
    else
      k_true_residual3<4, float><<<PT, RED_T, 0, st>>>(A->n, A->rowptr, A->colidx,
                                                        (const float *)A->vals, x, b, r, part);
  } else {
    if (A->dtype == SG_F64)
      k_true_residual_any<double><<<PT, RED_T, 0, st>>>(A->n, A->bs, A->rowptr, A->colidx,
                                                         (const double *)A->vals, x, b, r, part);
    else
      k_true_residual_any<float><<<PT, RED_T, 0, st>>>(A->n, A->bs, A->rowptr, A->colidx,
                                                        (const float *)A->vals, x, b, r, part);
  }
  SG_CHECK_LAUNCH();
  k_sum_parts<<<1, RED_T, 0, st>>>(part, PT, dres);
  SG_CHECK_LAUNCH();
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, dres, 8, cudaMemcpyDeviceToHost, st));
  SG_CHECK_CUDA(cudaStreamSynchronize(st));
  *h_rr = *(double *)c->h_stage;
  return SG_OK;
}

int sg_solve(sg_ctx *h, const sg_matrix *A, const sg_solve_opts *o, const double *b, double *x,
             sg_solve_result *res) {
  sg_solver *s = nullptr;
  SG_TRY(sg_solver_create(h, A, o, &s));
  int rc = sg_solver_solve(s, b, x, res);
  sg_solver_destroy(s);
  return rc;
}

}  // extern "C"

namespace sg {

void dot_launch(Ctx *c, int64_t len, const double *a, const double *b, double *part,
                double *dres) {
  const int P = grid_for(c, len, RED_T, 4);
  k_dot2<<<P, RED_T, 0, c->stream>>>(len, a, b, part);
  k_sum_parts<<<1, RED_T, 0, c->stream>>>(part, P, dres);
}

// Matrix-dependent data: the FP32 bulk copy (mixed, FP64 input) and the
// (block-)Jacobi inverse diagonal.  Re-run after the matrix values change.
int refresh_matrix(Solver *S) {
  Ctx *c = S->c;
  const sg_matrix *A = &S->A;
  const size_t vt = S->kind == KIND_MIXED ? 4 : 8;
  S->bulk_vals = A->vals;
  if (S->kind == KIND_MIXED && A->dtype == SG_F64) {
    const int64_t nv = A->nnzb * A->bs * A->bs;
    k_f64_to_f32<<<grid_for(c, nv, 256, 8), 256, 0, c->stream>>>(nv, (const double *)A->vals,
                                                                 (float *)S->vals32);
    SG_CHECK_LAUNCH();
    S->bulk_vals = S->vals32;
  }
  if (S->sym) SG_TRY(sym_fill(S->sym, c->stream, (const float *)S->bulk_vals));
  if (S->prec == PK_JACOBI || S->prec == PK_BLOCK3) {
    const int blk = S->prec == PK_BLOCK3;
    const int g = grid_for(c, A->n, 256, 8);
    if (vt == 4) {  // mixed: block inverses packed as 6 values (K2 and k_prec_dot read them so)
      if (A->dtype == SG_F64)
        k_diag_inv<double, float, true><<<g, 256, 0, c->stream>>>(
            A->n, A->bs, A->rowptr, A->colidx, (const double *)A->vals, (float *)S->dinv, blk,
            c->d_err);
      else
        k_diag_inv<float, float, true><<<g, 256, 0, c->stream>>>(
            A->n, A->bs, A->rowptr, A->colidx, (const float *)A->vals, (float *)S->dinv, blk,
            c->d_err);
    } else {
      if (A->dtype == SG_F64)
        k_diag_inv<double, double><<<g, 256, 0, c->stream>>>(A->n, A->bs, A->rowptr, A->colidx,
                                                             (const double *)A->vals,
                                                             (double *)S->dinv, blk, c->d_err);
      else
        k_diag_inv<float, double><<<g, 256, 0, c->stream>>>(A->n, A->bs, A->rowptr, A->colidx,
                                                            (const float *)A->vals,
                                                            (double *)S->dinv, blk, c->d_err);
    }
    SG_CHECK_LAUNCH();
    SG_TRY(check_device_error(c, "solver (diagonal)"));
  }
  if (S->prec == PK_EXTERNAL && S->ext) SG_TRY(learned_refresh(S));
  return SG_OK;
}

int solver_init(Ctx *c, const sg_matrix *A, const sg_solve_opts *o_in, Solver *S,
                int (*ext_setup)(Solver *)) {
  // SG_LANES_AUTOTUNE: the SpMV schedule the tuner finds fastest on this
  // matrix (the iteration's vectors: FP32 in mixed precision, else FP64)
  sg_solve_opts o_tuned = *o_in;
  const sg_solve_opts *o = &o_tuned;
  if (o_tuned.lanes == SG_LANES_AUTOTUNE) {
    o_tuned.lanes = 0;
    const int xdt = o_in->precision == SG_SOLVE_MIXED ? SG_F32 : SG_F64;
    if (!(xdt == SG_F32 && A->dtype == SG_F64)) {  // the bulk is A itself
      int32_t g = 0;
      float ms = 0.f;
      SG_TRY(sg_tune_spmv(reinterpret_cast<sg_ctx *>(c), A, xdt, 10, 0, &g, &ms, nullptr,
                          nullptr, nullptr, nullptr, 0));
      o_tuned.lanes = g;
    }
  }
  S->c = c;
  ctx_retain(c);
  S->A = *A;
  S->o = *o;
  if (S->o.batch <= 0) S->o.batch = 32;
  S->batch = (S->o.batch + 1) & ~1;
  S->len = (int64_t)A->n * A->bs;
  S->G = o->lanes > 0 ? o->lanes : default_lanes(A->n, A->nnzb, A->bs);
  if (S->G < 1 || S->G > 32 || (S->G & (S->G - 1))) S->G = default_lanes(A->n, A->nnzb, A->bs);
  if (A->bs != 3 && A->bs != 1) S->G = 1;
  S->P1 = grid_for(c, (int64_t)A->n * (A->bs == 3 || A->bs == 1 ? S->G : 1), RED_T, 8);
  S->P2 = grid_for(c, S->len, RED_T, 3);  // K2 holds 3 CTAs per SM
  S->prec = o->precond == SG_PRECOND_JACOBI ? PK_JACOBI
            : o->precond == SG_PRECOND_BLOCK_JACOBI ? PK_BLOCK3
            : o->precond == SG_PRECOND_LEARNED ? PK_EXTERNAL : PK_NONE;
  if (o->precision == SG_SOLVE_MIXED) S->kind = KIND_MIXED;
  else S->kind = A->dtype == SG_F64 ? KIND_F64 : KIND_F64_M32;
  const size_t vt = S->kind == KIND_MIXED ? 4 : 8;
  // K1: the TMA-staged kernel for 3x3 or scalar blocks with 16-byte aligned
  // arrays (unless a lane count is forced), else G lanes per row.
  const bool aligned = ((uintptr_t)A->vals % 16 == 0) && ((uintptr_t)A->colidx % 16 == 0);
  if ((A->bs == 3 || A->bs == 1) && aligned &&
      (o->lanes < 0 || (o->lanes == 0 && S->kind != KIND_F64))) {
    SG_TRY(cached_stats(c, A->n, A->rowptr, &S->pstats, true));
    S->maxrow = S->pstats.maxrow;
    S->tma_var = o->lanes < 0 ? -o->lanes - 1 : default_tma_variant(A->bs);
    const int vdt = (S->kind == KIND_F64) ? SG_F64 : SG_F32;
    const int xdt = S->kind == KIND_MIXED ? SG_F32 : SG_F64;
    int grid = 0;
    if (bsr3_tma_config(c, A->bs, vdt, xdt, S->tma_var, 1, A->n, S->pstats, &grid,
                        &S->tma_smem) ==
        SG_OK) {
      S->tma = 1;
      S->P1 = grid;
    }
  }
  if (o->storage == SG_STORAGE_SYMMETRIC) {
    SG_REQUIRE(A->bs == 3 && S->kind == KIND_MIXED,
               "sg_solver_create: symmetric storage needs bs = 3 and SG_SOLVE_MIXED");
    S->sym = new SymBsr();
    SG_TRY(sym_create(c, A->n, A->rowptr, A->colidx, A->nnzb, 0, S->sym));
    S->tma = 1;  // K1 leaves the finished p.q in ctl, as the TMA kernels do
    S->P1 = S->sym->grid[1];
  }
  const int np = S->P1 > S->P2 ? S->P1 : S->P2;
  SG_TRY(alloc_dev(S, (void **)&S->ctl, sizeof(SolveCtl)));
  SG_CHECK_CUDA(cudaMallocHost((void **)&S->hctl, sizeof(SolveCtl)));
  SG_TRY(alloc_dev(S, &S->r, S->len * vt));
  SG_TRY(alloc_dev(S, &S->p, S->len * vt));
  SG_TRY(alloc_dev(S, &S->q, S->len * vt));
  SG_TRY(alloc_dev(S, &S->z, S->len * vt));
  SG_TRY(alloc_dev(S, (void **)&S->xw, S->len * 8));
  SG_TRY(alloc_dev(S, (void **)&S->rhi, S->len * 8));
  SG_TRY(alloc_dev(S, (void **)&S->part1, (size_t)np * 8));
  SG_TRY(alloc_dev(S, (void **)&S->part2, (size_t)np * 3 * 8));
  SG_TRY(alloc_dev(S, (void **)&S->part3, (size_t)np * 8));
  SG_TRY(alloc_dev(S, (void **)&S->dres, 64));
  if (S->kind == KIND_MIXED) {
    SG_TRY(alloc_dev(S, &S->xlo, S->len * 4));
    S->xupd = S->xlo;
  } else {
    S->xupd = S->xw;
  }
  if (S->kind == KIND_MIXED && A->dtype == SG_F64)
    SG_TRY(alloc_dev(S, &S->vals32, A->nnzb * A->bs * A->bs * 4));
  if (S->kind == KIND_MIXED && A->dtype == SG_F32 && A->bs == 3)
    SG_TRY(alloc_dev(S, (void **)&S->xsplit, S->len * 8));
  if (S->prec == PK_JACOBI || S->prec == PK_BLOCK3)
    SG_TRY(alloc_dev(S, &S->dinv,
                     (S->prec == PK_BLOCK3 ? (int64_t)A->n * 9 : S->len) * vt));
  SG_TRY(refresh_matrix(S));
  if (ext_setup) SG_TRY(ext_setup(S));
  switch (S->kind) {
    case KIND_F64: return capture_batch<double, double, double>(S);
    case KIND_F64_M32: return capture_batch<float, double, double>(S);
    default: return capture_batch<float, float, float>(S);
  }
}

int solver_solve(Solver *S, const double *b, double *x, sg_solve_result *res) {
  switch (S->kind) {
    case KIND_F64: return solve_impl<double, double, double>(S, b, x, res);
    case KIND_F64_M32: return solve_impl<float, double, double>(S, b, x, res);
    default: return solve_impl<float, float, float>(S, b, x, res);
  }
}

void solver_free(Solver *S) {
  if (!S) return;
  if (S->c) cudaStreamSynchronize(S->c->stream);
  if (S->gexec) cudaGraphExecDestroy(S->gexec);
  for (void *p : S->allocs) cudaFree(p);
  if (S->hctl) cudaFreeHost(S->hctl);
  if (S->ext_free) S->ext_free(S);
  if (S->sym) {
    sym_free(S->sym);
    delete S->sym;
  }
  if (S->c) ctx_release(S->c);
  delete S;
}

}  // namespace sg
