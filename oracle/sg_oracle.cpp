// ORACLE — test infrastructure, never part of the product.
//
// A plain-C++ CPU restatement of the Simit sparse-system hot path, used only
// by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
// checker.  The product (simit_gb300/) never links or calls it.
//
// Parity pins:
//   * pattern + slot map: pinned bit-exactly against the reference's own
//     PathIndexBuilder and runtime `loc` compiled from its sources
//     (oracle/build_ref.sh -> oracle/_ref/libref_pattern.so);
//   * assembly + blocked SpMV + CG: pinned against the golden values of the
//     reference's tests (test/program-isprings.cpp, test/program-cg-test.cpp,
//     test/program-fem-test.cpp) reproduced through this file;
//   * the P1 heat element and the 5-tet lattice forms have no reference test:
//     they are pinned only by this restatement.
//
// Every loop follows the loop nests the reference's lowering emits (printed
// with ir::lower for apps/springs/isprings.sim and apps/fem/fem_linear.sim):
//   element loop in ascending element order, `+=` into CSR slots found by a
//   linear search, zero-initialised outputs, BSR SpMV rows ascending / blocks
//   ascending / per block-row dot over the block columns then `+=`, and dot
//   products as a per-vertex partial sum added to the total.
// Compile with -ffp-contract=off: the reference JIT does not fuse multiply-adds.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <vector>

typedef int32_t i32;
typedef int64_t i64;
typedef uint32_t u32;

namespace {

// src/runtime.cpp:19-23 (`loc`): linear search of a row for a column.
inline u32 loc(i32 v0, i32 v1, const u32 *rowptr, const u32 *colidx) {
  u32 l = rowptr[v0];
  while ((i32)colidx[l] != v1) ++l;
  return l;
}

// src/runtime.cpp:90-94 (det3_f64)
template <typename T> T det3(const T *a) {
  return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
         a[2] * (a[3] * a[7] - a[4] * a[6]);
}

// src/runtime.cpp:147-173 (inv3_f64): cofactors, one reciprocal, products.
template <typename T> void inv3(const T *a, T *inv) {
  T cof00 = a[4] * a[8] - a[5] * a[7];
  T cof01 = -a[3] * a[8] + a[5] * a[6];
  T cof02 = a[3] * a[7] - a[4] * a[6];
  T cof10 = -a[1] * a[8] + a[2] * a[7];
  T cof11 = a[0] * a[8] - a[2] * a[6];
  T cof12 = -a[0] * a[7] + a[1] * a[6];
  T cof20 = a[1] * a[5] - a[2] * a[4];
  T cof21 = -a[0] * a[5] + a[2] * a[3];
  T cof22 = a[0] * a[4] - a[1] * a[3];
  T determ = a[0] * cof00 + a[1] * cof01 + a[2] * cof02;
  determ = T(1.0) / determ;
  inv[0] = cof00 * determ; inv[1] = cof10 * determ; inv[2] = cof20 * determ;
  inv[3] = cof01 * determ; inv[4] = cof11 * determ; inv[5] = cof21 * determ;
  inv[6] = cof02 * determ; inv[7] = cof12 * determ; inv[8] = cof22 * determ;
}

// Dense 3x3 product C = A*B with the reduction index ascending from zero
// (the lowered `(i,j A(i,+k)*B(+k,j))`).
template <typename T> void mm3(const T *A, const T *B, T *C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T t = 0;
      for (int k = 0; k < 3; ++k) t += A[i * 3 + k] * B[k * 3 + j];
      C[i * 3 + j] = t;
    }
}
template <typename T> void tr3(const T *A, T *At) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) At[i * 3 + j] = A[j * 3 + i];
}

// Lowered BSR SpMV (src/lower/index_expressions/lower_indexexprs.cpp:630-660):
//   y = 0; for q: for qp in row q: p = sinks[qp];
//     for q1: t = 0; for p1: t += A[qp*bs*bs + q1*bs + p1] * x[p*bs + p1];
//             y[q*bs + q1] += t
template <typename T>
void spmv(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx, const T *A,
          const T *x, T *y) {
  const i64 bb = (i64)bs * bs;
  for (i64 i = 0; i < (i64)n * bs; ++i) y[i] = 0;
  for (i32 q = 0; q < n; ++q)
    for (u32 qp = rowptr[q]; qp < rowptr[q + 1]; ++qp) {
      const i64 p = colidx[qp];
      for (i32 q1 = 0; q1 < bs; ++q1) {
        T t = 0;
        for (i32 p1 = 0; p1 < bs; ++p1)
          t += A[qp * bb + q1 * bs + p1] * x[p * bs + p1];
        y[(i64)q * bs + q1] += t;
      }
    }
}

// Lowered dot product over a blocked vector: per-vertex partial then total.
template <typename T> T dot(i32 n, i32 bs, const T *a, const T *b) {
  T s = 0;
  for (i32 q = 0; q < n; ++q) {
    T t = 0;
    for (i32 k = 0; k < bs; ++k) t += a[(i64)q * bs + k] * b[(i64)q * bs + k];
    s += t;
  }
  return s;
}

// The CG loop of apps/springs/isprings.sim:77-93, apps/fem/fem_linear.sim:
// 211-230 and test/input/program/femTet.sim (main): stop when r'r <= tol2
// or after maxiters.  x holds the initial guess on entry.
template <typename T>
int cg_normr2(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx, const T *A,
              const T *b, T *x, T tol2, int maxiters, T *normr2_out) {
  const i64 N = (i64)n * bs;
  std::vector<T> r(N), p(N), Ap(N);
  spmv(n, bs, rowptr, colidx, A, x, Ap.data());
  for (i64 i = 0; i < N; ++i) r[i] = b[i] - Ap[i];
  for (i64 i = 0; i < N; ++i) p[i] = r[i];
  int iter = 0;
  T normr2 = dot(n, bs, r.data(), r.data());
  while (normr2 > tol2 && iter < maxiters) {
    spmv(n, bs, rowptr, colidx, A, p.data(), Ap.data());
    T denom = dot(n, bs, p.data(), Ap.data());
    T alpha = normr2 / denom;
    for (i64 i = 0; i < N; ++i) x[i] = x[i] + alpha * p[i];
    T normr2old = normr2;
    for (i64 i = 0; i < N; ++i) r[i] = r[i] - alpha * Ap[i];
    normr2 = dot(n, bs, r.data(), r.data());
    T beta = normr2 / normr2old;
    for (i64 i = 0; i < N; ++i) p[i] = r[i] + beta * p[i];
    iter = iter + 1;
  }
  if (normr2_out) *normr2_out = normr2;
  return iter;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Pattern and slot map
// ---------------------------------------------------------------------------

// Restates PathIndexBuilder::buildSegmented for the assembly expression
// ∃e∈E.(v-e ∧ e-u) (src/path_indices.cpp:359-429 over Link::ve 248-276 and
// Link::ev 205-247, packed by 172-203): row v = ordered set of every endpoint
// of every edge incident on v; vertices without edges get empty rows.
// Returns nnz, or -1 if `cap` is too small.
i64 or_pattern(i32 n, const i32 *ep, i64 nE, i32 card, u32 *rowptr,
               u32 *colidx, i64 cap) {
  std::vector<std::vector<u32>> ve(n);
  for (i64 e = 0; e < nE; ++e)
    for (i32 i = 0; i < card; ++i) ve[ep[e * card + i]].push_back((u32)e);
  std::map<u32, std::set<u32>> rows;
  for (i32 v = 0; v < n; ++v) {
    std::set<u32> &s = rows[(u32)v];
    for (u32 e : ve[v])
      for (i32 j = 0; j < card; ++j) s.insert((u32)ep[(i64)e * card + j]);
  }
  i64 k = 0;
  for (auto &kv : rows) {
    rowptr[kv.first] = (u32)k;
    for (u32 c : kv.second) {
      if (k >= cap) return -1;
      colidx[k++] = c;
    }
  }
  rowptr[n] = (u32)k;
  return k;
}

// Element-to-slot map in gatherVVLocs order (src/inline.cpp:544-552):
// slots[(e*card + i)*card + j] = loc(ep[e,i], ep[e,j]).
void or_slots(const i32 *ep, i64 nE, i32 card, const u32 *rowptr,
              const u32 *colidx, u32 *slots) {
  for (i64 e = 0; e < nE; ++e)
    for (i32 i = 0; i < card; ++i)
      for (i32 j = 0; j < card; ++j)
        slots[(e * card + i) * card + j] =
            loc(ep[e * card + i], ep[e * card + j], rowptr, colidx);
}

// ---------------------------------------------------------------------------
// Blocked SpMV, dot, CG
// ---------------------------------------------------------------------------
void or_spmv_f64(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx,
                 const double *A, const double *x, double *y) {
  spmv<double>(n, bs, rowptr, colidx, A, x, y);
}
void or_spmv_f32(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx,
                 const float *A, const float *x, float *y) {
  spmv<float>(n, bs, rowptr, colidx, A, x, y);
}
double or_dot_f64(i32 n, i32 bs, const double *a, const double *b) {
  return dot<double>(n, bs, a, b);
}

int or_cg_normr2_f64(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx,
                     const double *A, const double *b, double *x, double tol2,
                     int maxiters, double *normr2_out) {
  return cg_normr2<double>(n, bs, rowptr, colidx, A, b, x, tol2, maxiters,
                           normr2_out);
}

// Jacobi-preconditioned CG of apps/thermal/thermal.sim:102-130 with a
// relative tolerance (tol^2 * b'b) and the true residual b - A*x recomputed
// every `refresh` iterations (thermal.sim uses 50).  The preconditioner is
// point Jacobi on the scalar diagonal of the blocked matrix.  Returns the
// iteration count; *relres_out = ||b - A x|| / ||b|| recomputed at exit.
// zr_stop = 1 keeps thermal.sim's second loop condition (z'r > tol^2 b'b).
int or_jacobi_pcg_f64(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx,
                      const double *A, const double *b, double *x, double tol,
                      int maxiters, int refresh, int zr_stop, double *relres_out) {
  const i64 N = (i64)n * bs, bb = (i64)bs * bs;
  std::vector<double> dinv(N), r(N), z(N), p(N), Ap(N);
  for (i32 q = 0; q < n; ++q) {
    const u32 l = loc(q, q, rowptr, colidx);
    for (i32 k = 0; k < bs; ++k)
      dinv[(i64)q * bs + k] = 1.0 / A[l * bb + k * bs + k];
  }
  spmv<double>(n, bs, rowptr, colidx, A, x, Ap.data());
  for (i64 i = 0; i < N; ++i) r[i] = b[i] - Ap[i];
  for (i64 i = 0; i < N; ++i) z[i] = dinv[i] * r[i];
  for (i64 i = 0; i < N; ++i) p[i] = z[i];
  int iter = 0;
  double rsold = dot<double>(n, bs, z.data(), r.data());
  const double bb2 = dot<double>(n, bs, b, b);
  const double tol2 = tol * tol * bb2;
  double nr = dot<double>(n, bs, r.data(), r.data());
  while (nr > tol2 && (!zr_stop || rsold > tol2) && iter < maxiters) {
    iter = iter + 1;
    spmv<double>(n, bs, rowptr, colidx, A, p.data(), Ap.data());
    double alpha = rsold / dot<double>(n, bs, Ap.data(), p.data());
    for (i64 i = 0; i < N; ++i) x[i] = x[i] + alpha * p[i];
    if (refresh <= 0 || iter % refresh != 0) {
      for (i64 i = 0; i < N; ++i) r[i] = r[i] - alpha * Ap[i];
    } else {
      spmv<double>(n, bs, rowptr, colidx, A, x, Ap.data());
      for (i64 i = 0; i < N; ++i) r[i] = b[i] - Ap[i];
    }
    for (i64 i = 0; i < N; ++i) z[i] = dinv[i] * r[i];
    double rsnew = dot<double>(n, bs, z.data(), r.data());
    for (i64 i = 0; i < N; ++i) p[i] = z[i] + (rsnew / rsold) * p[i];
    rsold = rsnew;
    nr = dot<double>(n, bs, r.data(), r.data());
  }
  if (relres_out) {
    spmv<double>(n, bs, rowptr, colidx, A, x, Ap.data());
    double s = 0;
    for (i64 i = 0; i < N; ++i) s += (b[i] - Ap[i]) * (b[i] - Ap[i]);
    *relres_out = std::sqrt(s) / std::sqrt(bb2);
  }
  return iter;
}

// ---------------------------------------------------------------------------
// Springs: apps/springs/isprings.sim (timestep), lowered form
// ---------------------------------------------------------------------------

// compute_mass_damping over points (isprings.sim:21-32) and compute_elasticity
// over springs (isprings.sim:34-68), then MDK = MD + K and f = fmg + fe.
// Outputs the BSR 3x3 values of MDK (on the spring pattern) and f[n*3].
void or_springs_assemble(int form, i32 n, const double *x, const double *v,
                         const double *m, const uint8_t *fixed, i64 nS,
                         const i32 *ep, const double *k, const double *l0,
                         double h, double viscous, const double *grav,
                         const u32 *rowptr, const u32 *colidx, double *MDK,
                         double *f) {
  const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  const i64 nnz = rowptr[n];
  std::vector<double> MD((i64)n * 9, 0.0), fmg((i64)n * 3, 0.0),
      K(nnz * 9, 0.0), fe((i64)n * 3, 0.0);
  for (i32 p = 0; p < n; ++p) {
    double mass = m[p];
    if (fixed[p]) {
      MD[(i64)p * 9] += 1;  // a scalar written to a block touches (0,0) only
    } else {
      double s0 = mass + (h * viscous);
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) MD[(i64)p * 9 + i * 3 + j] += s0 * I[i * 3 + j];
      double s1 = h * mass;
      for (int mm = 0; mm < 3; ++mm)
        fmg[(i64)p * 3 + mm] += (mass * v[(i64)p * 3 + mm]) + (s1 * grav[mm]);
    }
  }
  for (i64 s = 0; s < nS; ++s) {
    const i32 e0 = ep[2 * s], e1 = ep[2 * s + 1];
    u32 locs[4];
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        locs[i * 2 + j] = loc(ep[2 * s + i], ep[2 * s + j], rowptr, colidx);
    double stiffness = k[s];
    double dx[3];
    for (int q = 0; q < 3; ++q) dx[q] = x[(i64)e1 * 3 + q] - x[(i64)e0 * 3 + q];
    double nrm = 0, nt = 0;
    for (int q = 0; q < 3; ++q) nt += dx[q] * dx[q];
    nrm += nt;
    double l = std::sqrt(nrm);
    double fe0[3], kk[9];
    if (form == 0) {
      // apps/springs/isprings.sim:34-68
      double U[3];
      for (int q = 0; q < 3; ++q) U[q] = dx[q] / l;
      double f0 = stiffness * (l - l0[s]);
      double s2 = h * f0;
      for (int q = 0; q < 3; ++q) fe0[q] = s2 * U[q];
      double UUt[9], t6[9];
      for (int t = 0; t < 3; ++t)
        for (int u = 0; u < 3; ++u) UUt[t * 3 + u] = U[t] * U[u];
      double s3 = stiffness - (f0 / l), s4 = f0 / l, s5 = h * h;
      for (int j = 0; j < 3; ++j)
        for (int q = 0; q < 3; ++q)
          t6[j * 3 + q] = (s3 * UUt[j * 3 + q]) + (s4 * I[j * 3 + q]);
      for (int j = 0; j < 9; ++j) kk[j] = s5 * t6[j];
    } else {
      // test/input/program/isprings.sim (compute_elasticity):
      //   fe0 = h*stiffness/(l0*l0)*(l-l0)*dx/l
      //   k = h*h*stiffness/(l0*l0*l*l)*(dxdxt + (l-l0)/l*(dxtdx*I - dxdxt))
      const double L0 = l0[s];
      double sc = ((h * stiffness) / (L0 * L0)) * (l - L0);
      for (int q = 0; q < 3; ++q) fe0[q] = (sc * dx[q]) / l;
      double dxtdx = 0, dt = 0;
      for (int q = 0; q < 3; ++q) dt += dx[q] * dx[q];
      dxtdx += dt;
      double dxdxt[9];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) dxdxt[a * 3 + b] = dx[a] * dx[b];
      double cc = ((h * h) * stiffness) / (((L0 * L0) * l) * l);
      double rr = (l - L0) / l;
      for (int q = 0; q < 9; ++q)
        kk[q] = cc * (dxdxt[q] + (rr * ((dxtdx * I[q]) - dxdxt[q])));
    }
    if (!fixed[e0])
      for (int q = 0; q < 3; ++q) fe[(i64)e0 * 3 + q] += fe0[q];
    if (!fixed[e1])
      for (int q = 0; q < 3; ++q) fe[(i64)e1 * 3 + q] += -fe0[q];
    if (!fixed[e0] && !fixed[e1]) {
      for (int q = 0; q < 9; ++q) K[(i64)locs[0] * 9 + q] += kk[q];
      for (int q = 0; q < 9; ++q) K[(i64)locs[1] * 9 + q] += -kk[q];
      for (int q = 0; q < 9; ++q) K[(i64)locs[2] * 9 + q] += -kk[q];
      for (int q = 0; q < 9; ++q) K[(i64)locs[3] * 9 + q] += kk[q];
    } else {
      if (!fixed[e0])
        for (int q = 0; q < 9; ++q) K[(i64)locs[0] * 9 + q] += kk[q];
      if (!fixed[e1])
        for (int q = 0; q < 9; ++q) K[(i64)locs[3] * 9 + q] += kk[q];
    }
  }
  // MDK = MD + K (lowered: MDK = 0; MDK[loc(l,l)] = MD[l]; MDK[lm] += K[lm])
  for (i64 i = 0; i < nnz * 9; ++i) MDK[i] = 0;
  for (i32 l = 0; l < n; ++l) {
    const u32 d = loc(l, l, rowptr, colidx);
    for (int q = 0; q < 9; ++q) MDK[(i64)d * 9 + q] = MD[(i64)l * 9 + q];
    for (u32 lm = rowptr[l]; lm < rowptr[l + 1]; ++lm)
      for (int q = 0; q < 9; ++q)
        MDK[(i64)lm * 9 + q] = MDK[(i64)lm * 9 + q] + K[(i64)lm * 9 + q];
  }
  for (i64 i = 0; i < (i64)n * 3; ++i) f[i] = fmg[i] + fe[i];
}

// One isprings timestep (form 0: apps/springs/isprings.sim timestep; form 1:
// test/input/program/isprings.sim main): assemble, CG on MDK v = f from the current v
// (normr2 tolerance, maxiters), then x = x + h*v.  Returns CG iterations.
int or_springs_step(int form, i32 n, double *x, double *v, const double *m,
                    const uint8_t *fixed, i64 nS, const i32 *ep,
                    const double *k, const double *l0, double h,
                    double viscous, const double *grav, const u32 *rowptr,
                    const u32 *colidx, double tol2, int maxiters) {
  std::vector<double> MDK((i64)rowptr[n] * 9), f((i64)n * 3);
  or_springs_assemble(form, n, x, v, m, fixed, nS, ep, k, l0, h, viscous, grav,
                      rowptr, colidx, MDK.data(), f.data());
  int it = cg_normr2<double>(n, 3, rowptr, colidx, MDK.data(), f.data(), v,
                             tol2, maxiters, nullptr);
  for (i64 i = 0; i < (i64)n * 3; ++i) x[i] = x[i] + (h * v[i]);
  return it;
}

// ---------------------------------------------------------------------------
// test/input/program/cg.sim: scalar spring Laplacian A = I - c*K, norm-based CG
// ---------------------------------------------------------------------------

// f over springs (cg.sim:13-18): A(p0,p0)=a, A(p0,p1)=-a, A(p1,p0)=-a,
// A(p1,p1)=a; eye over points; A = I + scale*K on K's pattern (scale=-0.01).
void or_scalar_springs_assemble(i32 n, i64 nS, const i32 *ep, const double *a,
                                double diag, double scale, const u32 *rowptr,
                                const u32 *colidx, double *A) {
  const i64 nnz = rowptr[n];
  std::vector<double> K(nnz, 0.0);
  for (i64 s = 0; s < nS; ++s) {
    u32 locs[4];
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        locs[i * 2 + j] = loc(ep[2 * s + i], ep[2 * s + j], rowptr, colidx);
    K[locs[0]] += a[s];
    K[locs[1]] += -a[s];
    K[locs[2]] += -a[s];
    K[locs[3]] += a[s];
  }
  for (i64 i = 0; i < nnz; ++i) A[i] = 0;
  for (i32 l = 0; l < n; ++l) {
    const u32 d = loc(l, l, rowptr, colidx);
    A[d] = diag;
    for (u32 lm = rowptr[l]; lm < rowptr[l + 1]; ++lm)
      A[lm] = A[lm] + (scale * K[lm]);
  }
}

// cg.sim:25-53: x = 0, stop when sqrt(r'r) <= tol or after maxiters.
int or_cg_norm_f64(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx,
                   const double *A, const double *b, double *x, double tol,
                   int maxiters) {
  const i64 N = (i64)n * bs;
  std::vector<double> r(N), p(N), Ap(N);
  for (i64 i = 0; i < N; ++i) x[i] = 0;
  spmv<double>(n, bs, rowptr, colidx, A, x, Ap.data());
  for (i64 i = 0; i < N; ++i) r[i] = b[i] - Ap[i];
  for (i64 i = 0; i < N; ++i) p[i] = r[i];
  int iter = 0;
  double normr = std::sqrt(dot<double>(n, bs, r.data(), r.data()));
  while (normr > tol && iter < maxiters) {
    spmv<double>(n, bs, rowptr, colidx, A, p.data(), Ap.data());
    double denom = dot<double>(n, bs, p.data(), Ap.data());
    double alpha = dot<double>(n, bs, r.data(), r.data()) / denom;
    for (i64 i = 0; i < N; ++i) x[i] = x[i] + alpha * p[i];
    double oldr = dot<double>(n, bs, r.data(), r.data());
    for (i64 i = 0; i < N; ++i) r[i] = r[i] - alpha * Ap[i];
    double newr = dot<double>(n, bs, r.data(), r.data());
    double beta = newr / oldr;
    for (i64 i = 0; i < N; ++i) p[i] = r[i] + beta * p[i];
    normr = std::sqrt(dot<double>(n, bs, r.data(), r.data()));
    iter = iter + 1;
  }
  return iter;
}

// ---------------------------------------------------------------------------
// Tetrahedral FEM: test/input/program/femTet.sim and apps/fem/fem_linear.sim
// ---------------------------------------------------------------------------

// precomputeTetMat (femTet.sim, fem_linear.sim:176-193): B = inv(Ds_rest),
// W = -(1/6) det(Ds_rest), m(v) += 0.25*rho*W.  B[nT*9], W[nT], m[n].
void or_tet_precompute(i32 n, const double *x, i64 nT, const i32 *tets,
                       double rho, double *B, double *W, double *m) {
  for (i32 i = 0; i < n; ++i) m[i] = 0;
  for (i64 t = 0; t < nT; ++t) {
    const i32 *v = tets + 4 * t;
    double M[9];
    for (int ii = 0; ii < 3; ++ii)
      for (int jj = 0; jj < 3; ++jj)
        M[jj * 3 + ii] = x[(i64)v[ii] * 3 + jj] - x[(i64)v[3] * 3 + jj];
    double Bi[9];
    inv3(M, Bi);
    for (int q = 0; q < 9; ++q) B[t * 9 + q] = 1.0 * Bi[q];
    double vol = -(1.0 / 6.0) * det3(M);
    W[t] = vol;
    for (int ii = 0; ii < 4; ++ii) m[v[ii]] += (0.25 * rho) * vol;
  }
}

namespace {
// Ds(jj,ii) = x_ii(jj) - x_3(jj); F = Ds * B
void tet_F(const double *x, const i32 *v, const double *B, double *F) {
  double Ds[9];
  for (int ii = 0; ii < 3; ++ii)
    for (int jj = 0; jj < 3; ++jj)
      Ds[jj * 3 + ii] = x[(i64)v[ii] * 3 + jj] - x[(i64)v[3] * 3 + jj];
  mm3(Ds, B, F);
}

// femTet.sim dPdF: dP = u*dF + (u - l*JJ)*Finv'*FidF' + l*trace(FidF)*Finv'
void neo_dPdF(double u, double l, const double *F, const double *dF,
              double *dP) {
  double JJ = std::log(det3(F));
  double Finv[9], FidF[9], FinvT[9], FidFT[9], s1[9], t2[9];
  inv3(F, Finv);
  mm3(Finv, dF, FidF);
  tr3(Finv, FinvT);
  tr3(FidF, FidFT);
  double c = u - l * JJ;
  for (int q = 0; q < 9; ++q) s1[q] = c * FinvT[q];
  mm3(s1, FidFT, t2);
  double trc = FidF[0] + FidF[4] + FidF[8];
  double c3 = l * trc;
  for (int q = 0; q < 9; ++q) dP[q] = ((u * dF[q]) + t2[q]) + (c3 * FinvT[q]);
}

// fem_linear.sim dPdF: dP = u*(dF + dF') + l*trace(dF)*I
void lin_dPdF(double u, double l, const double *dF, double *dP) {
  const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  double t = dF[0] + dF[4] + dF[8];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      dP[i * 3 + j] =
          (u * (dF[i * 3 + j] + dF[j * 3 + i])) + ((l * t) * I[i * 3 + j]);
}

// H = -W * P * B' : ((-W) * P) * B'
void tet_H(double W, const double *P, const double *B, double *H) {
  double s[9], Bt[9];
  for (int q = 0; q < 9; ++q) s[q] = (-W) * P[q];
  tr3(B, Bt);
  mm3(s, Bt, H);
}
}  // namespace

// compute_force (femTet.sim / fem_linear.sim:55-93).  `neo` selects the
// neo-Hookean PK1 (femTet) or the linear one (fem_linear).  u, l are per-tet.
// f[n*3] is zeroed then accumulated in element order.
void or_tet_force(int neo, i32 n, const double *x, const double *v,
                  const i32 *c, i64 nT, const i32 *tets, const double *B,
                  const double *W, const double *u, const double *l,
                  double h, double rho, const double *grav, double *f) {
  for (i64 i = 0; i < (i64)n * 3; ++i) f[i] = 0;
  for (i64 t = 0; t < nT; ++t) {
    const i32 *vv = tets + 4 * t;
    const double *Bt = B + 9 * t;
    double m = (0.25 * rho) * W[t];
    double fg[3];
    for (int q = 0; q < 3; ++q) fg[q] = m * grav[q];
    double F[9], P[9], H[9];
    tet_F(x, vv, Bt, F);
    if (neo) {
      // PK1: JJ = log(det F); Finv = inv(F)'; P = u*(F - Finv) + l*JJ*Finv
      double JJ = std::log(det3(F));
      double Fi[9], FinvT[9];
      inv3(F, Fi);
      tr3(Fi, FinvT);
      for (int q = 0; q < 9; ++q)
        P[q] = (u[t] * (F[q] - FinvT[q])) + ((l[t] * JJ) * FinvT[q]);
    } else {
      // PK1: FI = F - I; tr = trace(FI); P = u*(FI + FI') + l*tr*I
      const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
      double FI[9];
      for (int q = 0; q < 9; ++q) FI[q] = F[q] - I[q];
      double tr = (FI[0] + FI[4]) + FI[8];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          P[i * 3 + j] = (u[t] * (FI[i * 3 + j] + FI[j * 3 + i])) +
                         ((l[t] * tr) * I[i * 3 + j]);
    }
    tet_H(W[t], P, Bt, H);
    for (int ii = 0; ii < 3; ++ii) {
      double fi[3] = {H[0 * 3 + ii], H[1 * 3 + ii], H[2 * 3 + ii]};
      if (c[vv[ii]] <= 0)
        for (int q = 0; q < 3; ++q) f[(i64)vv[ii] * 3 + q] += h * fi[q];
      if (c[vv[3]] <= 0)
        for (int q = 0; q < 3; ++q) f[(i64)vv[3] * 3 + q] += (-h) * fi[q];
    }
    for (int ii = 0; ii < 4; ++ii)
      if (c[vv[ii]] <= 0)
        for (int q = 0; q < 3; ++q)
          f[(i64)vv[ii] * 3 + q] += (h * fg[q]) + (m * v[(i64)vv[ii] * 3 + q]);
  }
}

// compute_stiffness of femTet.sim (neo-Hookean, dPdF per column vertex `row`
// and direction kk) and of fem_linear.sim:105-174 (Ke = W*B'*E*B, linear) into
// BSR 3x3 values A on the tet pattern (zeroed first, element order).
void or_tet_stiffness(int neo, i32 n, const double *x, const i32 *c, i64 nT,
                      const i32 *tets, const double *B, const double *W,
                      const double *u, const double *l, double h, double rho,
                      const u32 *rowptr, const u32 *colidx, double *A) {
  const i64 nnz = rowptr[n];
  for (i64 i = 0; i < nnz * 9; ++i) A[i] = 0;
  for (i64 t = 0; t < nT; ++t) {
    const i32 *vv = tets + 4 * t;
    const double *Bt = B + 9 * t;
    u32 locs[16];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) locs[i * 4 + j] = loc(vv[i], vv[j], rowptr, colidx);
    if (neo) {
      double F[9];
      tet_F(x, vv, Bt, F);
      double dFRow[12];
      for (int ii = 0; ii < 3; ++ii) {
        for (int ll = 0; ll < 3; ++ll) dFRow[ii * 3 + ll] = Bt[ii * 3 + ll];
        dFRow[9 + ii] = -((Bt[0 * 3 + ii] + Bt[1 * 3 + ii]) + Bt[2 * 3 + ii]);
      }
      for (int row = 0; row < 4; ++row) {
        double Kb[4 * 9];  // Kb(jj, a, kk) at jj*9 + a*3 + kk
        for (int q = 0; q < 36; ++q) Kb[q] = 0;
        for (int kk = 0; kk < 3; ++kk) {
          double dF[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
          for (int ll = 0; ll < 3; ++ll) dF[kk * 3 + ll] = dFRow[row * 3 + ll];
          double dP[9], dH[9];
          neo_dPdF(u[t], l[t], F, dF, dP);
          tet_H(W[t], dP, Bt, dH);
          for (int ii = 0; ii < 3; ++ii) {
            for (int ll = 0; ll < 3; ++ll) Kb[ii * 9 + ll * 3 + kk] = dH[ll * 3 + ii];
            Kb[3 * 9 + ii * 3 + kk] =
                -((dH[ii * 3 + 0] + dH[ii * 3 + 1]) + dH[ii * 3 + 2]);
          }
        }
        for (int jj = 0; jj < 4; ++jj)
          if (c[vv[jj]] <= 0 && c[vv[row]] <= 0) {
            const u32 s = locs[jj * 4 + row];
            for (int q = 0; q < 9; ++q) A[(i64)s * 9 + q] += -((h * h) * Kb[jj * 9 + q]);
          }
      }
    } else {
      // E (6x6) isotropic; dN (4x3); strain-displacement Bm (6x12);
      // Ke = ((W * Bm') * E) * Bm.
      double E[36] = {0};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) E[i * 6 + j] = l[t];
      for (int i = 0; i < 3; ++i) E[i * 6 + i] = l[t] + 2.0 * u[t];
      for (int i = 3; i < 6; ++i) E[i * 6 + i] = u[t];
      double dN[12] = {0};
      for (int vi = 0; vi < 3; ++vi)
        for (int di = 0; di < 3; ++di) {
          dN[vi * 3 + di] = Bt[vi * 3 + di];
          dN[9 + di] = dN[9 + di] - Bt[vi * 3 + di];
        }
      double Bm[72] = {0};
      for (int vi = 0; vi < 4; ++vi) {
        for (int di = 0; di < 3; ++di) Bm[di * 12 + 3 * vi + di] = dN[vi * 3 + di];
        Bm[3 * 12 + 3 * vi] = dN[vi * 3 + 1];
        Bm[3 * 12 + 3 * vi + 1] = dN[vi * 3 + 0];
        Bm[4 * 12 + 3 * vi + 1] = dN[vi * 3 + 2];
        Bm[4 * 12 + 3 * vi + 2] = dN[vi * 3 + 1];
        Bm[5 * 12 + 3 * vi] = dN[vi * 3 + 2];
        Bm[5 * 12 + 3 * vi + 2] = dN[vi * 3 + 0];
      }
      double WBt[72], T[72], Ke[144];
      for (int r = 0; r < 12; ++r)
        for (int a = 0; a < 6; ++a) WBt[r * 6 + a] = W[t] * Bm[a * 12 + r];
      for (int r = 0; r < 12; ++r)
        for (int a = 0; a < 6; ++a) {
          double s = 0;
          for (int k = 0; k < 6; ++k) s += WBt[r * 6 + k] * E[k * 6 + a];
          T[r * 6 + a] = s;
        }
      for (int r = 0; r < 12; ++r)
        for (int cc = 0; cc < 12; ++cc) {
          double s = 0;
          for (int k = 0; k < 6; ++k) s += T[r * 6 + k] * Bm[k * 12 + cc];
          Ke[r * 12 + cc] = s;
        }
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
          if (c[vv[i]] <= 0 && c[vv[j]] <= 0) {
            const u32 s = locs[i * 4 + j];
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b)
                A[(i64)s * 9 + a * 3 + b] += (h * h) * Ke[(3 * i + a) * 12 + 3 * j + b];
          }
    }
    // M = m*I on each vertex's diagonal block, m = 0.25*rho*W
    double m = (0.25 * rho) * W[t];
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int ii = 0; ii < 4; ++ii) {
      const u32 s = locs[ii * 4 + ii];
      for (int q = 0; q < 9; ++q) A[(i64)s * 9 + q] += m * I[q];
    }
  }
}

// One femTet / fem_linear `main` step: f, A, CG from x = v (normr2 tolerance),
// v = x, x = h*x + x.  Returns the CG iteration count.
int or_tet_step(int neo, i32 n, double *x, double *v, const i32 *c, i64 nT,
                const i32 *tets, const double *B, const double *W,
                const double *u, const double *l, double h, double rho,
                const double *grav, const u32 *rowptr, const u32 *colidx,
                double tol2, int maxiters) {
  std::vector<double> f((i64)n * 3), A((i64)rowptr[n] * 9);
  or_tet_force(neo, n, x, v, c, nT, tets, B, W, u, l, h, rho, grav, f.data());
  or_tet_stiffness(neo, n, x, c, nT, tets, B, W, u, l, h, rho, rowptr, colidx,
                   A.data());
  std::vector<double> xs(v, v + (i64)n * 3);
  for (i64 i = 0; i < (i64)n * 3; ++i) xs[i] = 1.0 * xs[i];
  int it = cg_normr2<double>(n, 3, rowptr, colidx, A.data(), f.data(),
                             xs.data(), tol2, maxiters, nullptr);
  for (i64 i = 0; i < (i64)n * 3; ++i) v[i] = xs[i];
  for (i64 i = 0; i < (i64)n * 3; ++i) x[i] = (h * xs[i]) + x[i];
  return it;
}

// ---------------------------------------------------------------------------
// P1 heat (backward Euler): restated, no reference test pins it.
//   A_ij = W/20*(1+δij) + dt*kappa*W*(g_i . g_j), scalar blocks, element order;
//   b_i  = sum_e sum_j W/20*(1+δij) * T0_j.
// g_i = row i of B (i<3), g_3 = -(g_0+g_1+g_2) summed in that order.
// ---------------------------------------------------------------------------
void or_heat_assemble(i32 n, i64 nT, const i32 *tets, const double *B,
                      const double *W, const double *kappa, double dt,
                      const double *T0, const u32 *rowptr, const u32 *colidx,
                      double *A, double *b) {
  const i64 nnz = rowptr[n];
  for (i64 i = 0; i < nnz; ++i) A[i] = 0;
  for (i32 i = 0; i < n; ++i) b[i] = 0;
  for (i64 t = 0; t < nT; ++t) {
    const i32 *vv = tets + 4 * t;
    const double *Bt = B + 9 * t;
    double g[12];
    for (int d = 0; d < 3; ++d) {
      for (int i = 0; i < 3; ++i) g[i * 3 + d] = Bt[i * 3 + d];
      g[9 + d] = -((Bt[0 * 3 + d] + Bt[1 * 3 + d]) + Bt[2 * 3 + d]);
    }
    const double mw = W[t] / 20.0;
    const double kw = (dt * kappa[t]) * W[t];
    for (int i = 0; i < 4; ++i) {
      double bi = 0;
      for (int j = 0; j < 4; ++j) {
        const double mij = (i == j) ? 2.0 * mw : mw;
        const double gg = (g[i * 3] * g[j * 3] + g[i * 3 + 1] * g[j * 3 + 1]) +
                          g[i * 3 + 2] * g[j * 3 + 2];
        A[loc(vv[i], vv[j], rowptr, colidx)] += mij + kw * gg;
        bi += mij * T0[vv[j]];
      }
      b[vv[i]] += bi;
    }
  }
}

// System-matrix expression out = D + s*K on K's pattern, the lowered loop of
// `MDK = MD + K` (apps/springs/isprings.sim:74): MDK = 0; MDK[loc(l,l)] =
// D[l] (or ident*I); MDK[lm] = MDK[lm] + (s*K[lm]) over the row's slots.
// has_d = 0: no diagonal term.
}  // extern "C"
namespace {
template <typename T>
void add_diag(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx, const T *D,
                     T ident, int has_d, T s, const T *K, T *out) {
  const i64 bb = (i64)bs * bs, nnz = rowptr[n];
  std::vector<T> M((size_t)(nnz * bb), T(0));
  for (i32 l = 0; l < n; ++l) {
    if (has_d) {
      const u32 d = loc(l, l, rowptr, colidx);
      for (i64 q = 0; q < bb; ++q)
        M[(size_t)(d * bb + q)] = D ? D[(i64)l * bb + q] : (q / bs == q % bs ? ident : T(0));
    }
    for (u32 lm = rowptr[l]; lm < rowptr[l + 1]; ++lm)
      for (i64 q = 0; q < bb; ++q) {
        const T sk = s * K[(i64)lm * bb + q];
        M[(size_t)(lm * bb + q)] = M[(size_t)(lm * bb + q)] + sk;
      }
  }
  std::copy(M.begin(), M.end(), out);
}
}  // namespace
extern "C" {
void or_add_diag_f64(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx, const double *D,
                     double ident, int has_d, double s, const double *K, double *out) {
  add_diag<double>(n, bs, rowptr, colidx, D, ident, has_d, s, K, out);
}
void or_add_diag_f32(i32 n, i32 bs, const u32 *rowptr, const u32 *colidx, const float *D,
                     float ident, int has_d, float s, const float *K, float *out) {
  add_diag<float>(n, bs, rowptr, colidx, D, ident, has_d, s, K, out);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Cloth (apps/cloth/cloth.sim): triangle stretching over faces (card 3) and
// dihedral bending over hinges (card 4), the per-element quantities their
// initialisation precomputes, and one explicit step of its `main`.  Each
// vector is a 3-array; dot(a, b) = (a0*b0 + a1*b1) + a2*b2 and
// norm(a) = sqrt(dot(a, a)), as the lowered tensor reductions sum them.  No
// reference test pins these forms: the restatement is checked against the
// program's own text compiled on the host, and the GPU against it.
// ---------------------------------------------------------------------------
namespace {

inline double cdot(const double *a, const double *b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

// cloth.sim:1-5 (cross)
inline void ccross(const double *a, const double *b, double *r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

inline void csub(const double *a, const double *b, double *r) {
  for (int q = 0; q < 3; ++q) r[q] = a[q] - b[q];
}

// cloth.sim:31-38 (computeAngle): the dihedral angle at edge p1-p2 between
// the triangles (p1, p2, q1) and (p1, p2, q2).
double cloth_angle(const double *p1, const double *p2, const double *q1, const double *q2) {
  double ev[3], d1[3], d2[3], n1[3], n2[3], c[3];
  csub(p2, p1, ev);
  csub(q1, p1, d1);
  ccross(ev, d1, n1);
  csub(q2, p1, d2);
  ccross(d2, ev, n2);
  const double mag = std::sqrt(cdot(ev, ev));
  for (int q = 0; q < 3; ++q) ev[q] = ev[q] / mag;
  ccross(n1, n2, c);
  return std::atan2(cdot(c, ev), cdot(n1, n2));
}

// cloth.sim:115-140 (dihedralAngleDerivatives): d theta / d(p1, p2, q1, q2).
void cloth_angle_grad(const double *p1, const double *p2, const double *q1, const double *q2,
                      double *dp1, double *dp2, double *dq1, double *dq2) {
  double v11[3], v12[3], v21[3], v22[3], v[3], n1[3], n2[3];
  csub(q1, p2, v11);
  csub(q1, p1, v12);
  csub(q2, p2, v21);
  csub(q2, p1, v22);
  csub(p2, p1, v);
  ccross(v12, v, n1);
  ccross(v, v22, n2);
  const double n1n2 = cdot(n1, n1), n2n2 = cdot(n2, n2), vn = std::sqrt(cdot(v, v));
  if (vn < 1e-8 || n1n2 < 1e-8 || n2n2 < 1e-8) {
    for (int q = 0; q < 3; ++q) dp1[q] = dp2[q] = dq1[q] = dq2[q] = 0.0;
    return;
  }
  double m12[3], m22[3];
  for (int q = 0; q < 3; ++q) {
    m12[q] = -v12[q];
    m22[q] = -v22[q];
  }
  const double a11 = cdot(v11, v), a21 = cdot(v21, v), a12 = cdot(m12, v), a22 = cdot(m22, v);
  for (int q = 0; q < 3; ++q) {
    dq1[q] = (n1[q] * vn) / n1n2;
    dq2[q] = (n2[q] * vn) / n2n2;
    const double F11 = ((n1[q] * a11) / vn) / n1n2, F12 = ((n2[q] * a21) / vn) / n2n2;
    const double F21 = ((n1[q] * a12) / vn) / n1n2, F22 = ((n2[q] * a22) / vn) / n2n2;
    dp1[q] = F11 + F12;
    dp2[q] = F21 + F22;
  }
}

}  // namespace

extern "C" {

// cloth.sim:66-102 (precomputeFaceQuantities): per face the stretching
// matrix K (3x3, row-major) and the rest squared edge lengths, edge i running
// from vertex i to vertex i+1.  Edge vector u_c (c = 0, 1, 2) is the edge
// opposite vertex c: x2-x1, x0-x2, x1-x0.
void or_cloth_faces(const double *x, i64 nF, const i32 *faces, double *K, double *rest) {
  for (i64 f = 0; f < nF; ++f) {
    const double *p0 = x + 3 * (i64)faces[3 * f], *p1 = x + 3 * (i64)faces[3 * f + 1],
                 *p2 = x + 3 * (i64)faces[3 * f + 2];
    double ed[3][3], u[3][3], c[3];  // ed[c]: column c of edgeVectors(p0, p1, p2)
    csub(p1, p0, ed[0]);
    csub(p2, p1, ed[1]);
    csub(p0, p2, ed[2]);
    for (int q = 0; q < 3; ++q) {
      u[0][q] = ed[1][q];
      u[1][q] = ed[2][q];
      u[2][q] = ed[0][q];
    }
    ccross(u[2], u[1], c);
    const double A = 0.5 * std::sqrt(cdot(c, c));
    double *Kf = K + 9 * f;
    for (int i = 0; i < 3; ++i) {
      const int j = (i + 1) % 3, k = (i + 2) % 3;
      for (int l = i; l < 3; ++l) {
        const int m = (l + 1) % 3, n = (l + 2) % 3;
        const double e = cdot(u[k], u[m]) * cdot(u[j], u[n]) + cdot(u[k], u[n]) * cdot(u[j], u[m]);
        Kf[i * 3 + l] = e;
        Kf[l * 3 + i] = e;
      }
    }
    const double den = ((256.0 * A) * A) * A;
    for (int q = 0; q < 9; ++q) Kf[q] = Kf[q] / den;
    for (int i = 0; i < 3; ++i) rest[3 * f + i] = cdot(ed[i], ed[i]);
  }
}

// cloth.sim:105-113 (precomputeHingeQuantities): rest angle, rest length of
// the shared edge (vertices 0, 1) and 2 (A1 + A2) / (3 |e0|).
void or_cloth_hinges(const double *x, i64 nH, const i32 *hinges, double *angle, double *len,
                     double *perp) {
  for (i64 h = 0; h < nH; ++h) {
    const double *p[4];
    for (int a = 0; a < 4; ++a) p[a] = x + 3 * (i64)hinges[4 * h + a];
    angle[h] = cloth_angle(p[0], p[1], p[2], p[3]);
    double e[3], d2[3], d3[3], c2[3], c3[3];
    csub(p[1], p[0], e);
    csub(p[2], p[0], d2);
    csub(p[3], p[0], d3);
    ccross(e, d2, c2);
    ccross(e, d3, c3);
    const double A1 = 0.5 * std::sqrt(cdot(c2, c2)), A2 = 0.5 * std::sqrt(cdot(c3, c3));
    const double e0 = std::sqrt(cdot(e, e));
    perp[h] = (2.0 * (A1 + A2)) / (3.0 * e0);
    len[h] = e0;
  }
}

// cloth.sim:142-164 (stretchingForce, `map ... to faces reduce +`): per
// vertex k of a face, three terms (i = 0, 1, 2)
//   -4 (K(i,k+1) s_i v_{k+1} - K(i,k+2) s_i v_{k+2}),
// v_c the current edge opposite vertex c and s_i its squared length minus
// the rest one; f (3 per vertex) is zeroed, then faces in order add theirs.
void or_cloth_stretch(i32 n, const double *x, i64 nF, const i32 *faces, const double *K,
                      const double *rest, double *f) {
  for (i64 i = 0; i < (i64)n * 3; ++i) f[i] = 0.0;
  for (i64 e = 0; e < nF; ++e) {
    const i32 *vv = faces + 3 * e;
    const double *p0 = x + 3 * (i64)vv[0], *p1 = x + 3 * (i64)vv[1], *p2 = x + 3 * (i64)vv[2];
    double v[3][3];
    csub(p2, p1, v[0]);
    csub(p0, p2, v[1]);
    csub(p1, p0, v[2]);
    const double r[3] = {rest[3 * e + 1], rest[3 * e + 2], rest[3 * e + 0]};
    double s[3];
    for (int i = 0; i < 3; ++i) s[i] = cdot(v[i], v[i]) - r[i];
    const double *Ke = K + 9 * e;
    for (int k = 0; k < 3; ++k) {
      const int k2 = (k + 1) % 3, k1 = (k + 2) % 3;
      for (int i = 0; i < 3; ++i)
        for (int q = 0; q < 3; ++q) {
          const double t = (Ke[i * 3 + k2] * s[i]) * v[k2][q] - (Ke[i * 3 + k1] * s[i]) * v[k1][q];
          f[3 * (i64)vv[k] + q] += -4.0 * t;
        }
    }
  }
}

// cloth.sim:166-173 (bendingForce, `map ... to hinges reduce +`): per hinge
// vertex a, -d theta/d x_a * L / Lperp * (theta - theta_rest), one term.
void or_cloth_bend(i32 n, const double *x, i64 nH, const i32 *hinges, const double *angle,
                   const double *len, const double *perp, double *f) {
  for (i64 i = 0; i < (i64)n * 3; ++i) f[i] = 0.0;
  for (i64 h = 0; h < nH; ++h) {
    const double *p[4];
    for (int a = 0; a < 4; ++a) p[a] = x + 3 * (i64)hinges[4 * h + a];
    const double th = cloth_angle(p[0], p[1], p[2], p[3]);
    double d[4][3];
    cloth_angle_grad(p[0], p[1], p[2], p[3], d[0], d[1], d[2], d[3]);
    const double dth = th - angle[h];
    for (int a = 0; a < 4; ++a)
      for (int q = 0; q < 3; ++q)
        f[3 * (i64)hinges[4 * h + a] + q] += (((-d[a][q]) * len[h]) / perp[h]) * dth;
  }
}

// cloth.sim:201-222 (main) for one step of length dt: advance x by dt v,
// project points inside the radius-2 sphere at the origin onto it
// (cloth.sim:185-192, enforceConstraints, velocity corrected), then
//   F = ks stretch + kb bend - damping v,   v += dt (g + Minv F),
// Minv = diag(1/m) with 0 on fixed points (cloth.sim:175-183).  gravityForce
// (cloth.sim:194-199) writes (0, -9.8, 0) and, on a fixed point, (0, 0, 0)
// after it; writes to a map's result accumulate (src/lower/lower_maps.cpp:
// 38-47), so every point gets g = (0, -9.8, 0).  x, v (3 per point) are
// updated in place.
void or_cloth_step(i32 n, double *x, double *v, const double *m, const i32 *fixed, i64 nF,
                   const i32 *faces, const double *K, const double *rest, i64 nH,
                   const i32 *hinges, const double *angle, const double *len,
                   const double *perp, double dt, double ks, double kb, double damping) {
  const i64 n3 = (i64)n * 3;
  for (i64 i = 0; i < n3; ++i) x[i] = x[i] + dt * v[i];
  for (i32 p = 0; p < n; ++p) {
    double *xp = x + 3 * (i64)p, *vp = v + 3 * (i64)p;
    const double dist = std::sqrt(cdot(xp, xp));
    if (dist < 2.0) {
      double np[3];
      for (int q = 0; q < 3; ++q) np[q] = (2.0 * xp[q]) / dist;
      for (int q = 0; q < 3; ++q) vp[q] = vp[q] + (np[q] - xp[q]) / dt;
      for (int q = 0; q < 3; ++q) xp[q] = 1.0 * np[q];
    }
  }
  std::vector<double> fs(n3), fb(n3);
  or_cloth_stretch(n, x, nF, faces, K, rest, fs.data());
  or_cloth_bend(n, x, nH, hinges, angle, len, perp, fb.data());
  for (i64 i = 0; i < n3; ++i) {
    const double tot = (fs[i] * ks + fb[i] * kb) - damping * v[i];
    const i32 p = (i32)(i / 3);
    const double g = i % 3 == 1 ? -9.8 : 0.0;
    const double minv = fixed[p] > 0 ? 0.0 : 1.0 / m[p];
    v[i] = v[i] + dt * (g + minv * tot);
  }
}

}  // extern "C"
