"""Element functions written as CUDA C++ for `JitAssembly` (the contract of
sg_jit_assembly_create: `int element_block(e, i, j, ep, f, sg_block *blk)`
writes the terms element e adds to block (i, j) and returns their count).

Each one restates a map function of the reference's programs in the same
operation order as the precompiled kernel for it, so that the compiled
assembly gives the same values bit for bit:

* BLOCKS — block (i, j) read from a caller array [nE, card, card, bs, bs]
  (the generic `map f to E reduce +` of `sg_assemble_blocks`);
* heat(dt) — the P1 heat element, A_ij = W/20 (1 + d_ij) + (dt kappa W)
  g_i.g_j (fields B, W, kappa);
* linear_tet(h, rho) — the linear-elastic tetrahedron of fem_linear.sim
  (apps/fem/fem_linear.sim:95-174, the closed form of the precompiled
  kernel): h^2 W (lambda g_i g_j^T + mu g_j g_i^T +
  mu (g_i.g_j) I) where both vertices are free, then the lumped mass
  (rho/4) W I on the diagonal block as a second term (fields B, W, mu,
  lambda, and the int32 constraint flags c).
"""

BLOCKS = r"""
__device__ int element_block(long long e, int i, int j, const int *ep, const real *const *f,
                             sg_block *blk) {
  const real *b = f[0] + ((e * CARD + i) * CARD + j) * BS * BS;
  for (int a = 0; a < BS; ++a)
    for (int c = 0; c < BS; ++c) blk[0][a][c] = b[a * BS + c];
  return 1;
}
"""


def _lit(x):
    return "%.17g" % float(x)


def heat(dt):
    return r"""
__device__ void grad(const real *Bt, int i, real g[3]) {
  for (int d = 0; d < 3; ++d)
    g[d] = (i < 3) ? Bt[i * 3 + d] : -((Bt[0 * 3 + d] + Bt[1 * 3 + d]) + Bt[2 * 3 + d]);
}
__device__ int element_block(long long e, int i, int j, const int *ep, const real *const *f,
                             sg_block *blk) {
  const real *Bt = f[0] + 9 * e;
  real gi[3], gj[3];
  grad(Bt, i, gi);
  grad(Bt, j, gj);
  const real dt = (real)DT;
  const real mw = f[1][e] / real(20.0);
  const real kw = (dt * f[2][e]) * f[1][e];
  const real mij = (i == j) ? real(2.0) * mw : mw;
  const real gg = (gi[0] * gj[0] + gi[1] * gj[1]) + gi[2] * gj[2];
  blk[0][0][0] = mij + kw * gg;
  return 1;
}
""".replace("DT", _lit(dt))


def linear_tet(h, rho):
    return r"""
__device__ inline float mrn(float a, float b) { return __fmul_rn(a, b); }
__device__ inline double mrn(double a, double b) { return __dmul_rn(a, b); }
__device__ inline float arn(float a, float b) { return __fadd_rn(a, b); }
__device__ inline double arn(double a, double b) { return __dadd_rn(a, b); }
__device__ void dN(const real *Bt, int vi, real g[3]) {
  for (int d = 0; d < 3; ++d)
    g[d] = (vi < 3) ? Bt[vi * 3 + d] : ((real(0) - Bt[d]) - Bt[3 + d]) - Bt[6 + d];
}
// every product pairs a factor of vertex i with one of vertex j, without
// contraction: block (j, i) is bitwise the transpose of block (i, j)
__device__ int element_block(long long e, int i, int j, const int *ep, const real *const *f,
                             sg_block *blk) {
  const int *c = reinterpret_cast<const int *>(f[4]);
  const real W = f[1][e];
  int nt = 0;
  if (c[ep[i]] <= 0 && c[ep[j]] <= 0) {
    const real *Bt = f[0] + 9 * e;
    const real u = f[2][e], lm = f[3][e], h = (real)HSTEP;
    real gi[3], gj[3];
    dN(Bt, i, gi);
    dN(Bt, j, gj);
    const real gij = arn(arn(mrn(gi[0], gj[0]), mrn(gi[1], gj[1])), mrn(gi[2], gj[2]));
    const real hw = mrn(mrn(h, h), W);
    const real ug = mrn(u, gij);
    for (int l = 0; l < 3; ++l)
      for (int m = 0; m < 3; ++m) {
        real t = arn(mrn(lm, mrn(gi[l], gj[m])), mrn(u, mrn(gi[m], gj[l])));
        if (l == m) t = arn(t, ug);
        blk[0][l][m] = mrn(hw, t);
      }
    nt = 1;
  }
  if (i == j) {
    const real mm = (real(0.25) * (real)RHO) * W;
    for (int l = 0; l < 3; ++l)
      for (int m = 0; m < 3; ++m) blk[nt][l][m] = mm * real(l == m);
    ++nt;
  }
  return nt;
}
""".replace("HSTEP", _lit(h)).replace("RHO", _lit(rho))
