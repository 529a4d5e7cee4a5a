// Solver state shared by sg_solver.cu and the learned-preconditioner solver.
#pragma once
#include <vector>

#include "sg_internal.cuh"
#include "sg_solver_kernels.cuh"
#include "sg_spmv_api.h"

#include "sg_sym.h"

namespace sg {

struct Solver {
  Ctx *c = nullptr;
  sg_matrix A{};
  sg_solve_opts o{};
  int kind = 0;        // KIND_F64 / KIND_F64_M32 / KIND_MIXED
  int prec = 0;        // PrecKind
  int flexible = 0;    // Polak-Ribiere beta (variable preconditioner)
  int batch = 32;
  int64_t len = 0;     // n * bs
  int G = 4, P1 = 1, P2 = 1;
  int tma = 0, tma_var = 0, maxrow = 0;  // K1 uses the TMA-staged SpMV (variant)
  PatternStats pstats;
  size_t tma_smem = 0;
  int64_t launches = 0;             // kernels launched by the current solve
  int64_t graph_kernels = 0;        // kernel nodes in one batch graph
  const void *bulk_vals = nullptr;  // matrix values used by the iteration
  void *vals32 = nullptr;
  void *r = nullptr, *p = nullptr, *q = nullptr, *z = nullptr, *xlo = nullptr, *dinv = nullptr;
  void *xupd = nullptr;             // the x the iteration updates (xw or xlo)
  double *xw = nullptr, *rhi = nullptr;
  float *xsplit = nullptr;          // x_hi as floats xh | xl (compensated residual checks)
  double *part1 = nullptr, *part2 = nullptr, *part3 = nullptr, *dres = nullptr;
  SolveCtl *ctl = nullptr, *hctl = nullptr;
  cudaGraphExec_t gexec = nullptr;
  std::vector<void *> allocs;
  // External preconditioner hooks (learned preconditioner).  ext_prec runs
  // inside the captured iteration between K2 and K3 (par: the iteration's
  // parity slot): z = M(r) and the partials rr | rz | zq into part2, or,
  // with ext_decides, the iteration already decided in ctl (status, beta),
  // so that K3 only streams.  ext_prec_apply: z = M(r) and the partials of
  // r.z into part3 (set-up / restart).
  int (*ext_prec)(Solver *, cudaStream_t, int par) = nullptr;
  int ext_decides = 0;
  int (*ext_prec_apply)(Solver *, cudaStream_t) = nullptr;
  void (*ext_free)(Solver *) = nullptr;
  // ext_k2 (optional) replaces the iteration's K2 (the folded learned
  // iteration's r update and x = L^-1 r)
  int (*ext_k2)(Solver *, cudaStream_t, int par) = nullptr;
  // > 0: K3 sums this many partials per dot (the external preconditioner's
  // last kernel wrote them with its own grid), else P2
  int np2_ext = 0;
  // sg_solver_solve_ex: the FP64 copy of an FP32 right-hand side (allocated
  // on first use) and a zero initial guess for the current solve
  double *b64 = nullptr;
  int x_zero = 0;
  void *ext = nullptr;
  SymBsr *sym = nullptr;  // SG_STORAGE_SYMMETRIC: K1 reads the upper half
  int k3_xupd = 0;        // K3 applies x += alpha p (K2 = k_cg_update_w without x)
};

int default_lanes(int32_t n, int64_t nnzb, int32_t bs);
int solver_init(Ctx *c, const sg_matrix *A, const sg_solve_opts *o, Solver *S,
                int (*ext_setup)(Solver *));
int refresh_matrix(Solver *S);
int solver_solve(Solver *S, const double *b, double *x, sg_solve_result *res);
void solver_free(Solver *S);
int learned_refresh(Solver *S);
int learned_solver_init(Ctx *c, const sg_matrix *A, const sg_solve_opts *o, const float *params,
                        Solver *S);
void dot_launch(Ctx *c, int64_t len, const double *a, const double *b, double *part,
                double *dres);

}  // namespace sg
