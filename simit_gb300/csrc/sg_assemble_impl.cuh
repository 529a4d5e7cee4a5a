// Host launchers of the assembly kernels.  Included by sg_assemble_exact.cu
// (compiled with --fmad=false, namespace sg::exact) and sg_assemble_fast.cu
// (default contraction, namespace sg::fast); SG_ASM_NS names the namespace
// and SG_ASM_EXACT selects the operation-order-exact element forms.
#include "sg_assemble.cuh"
#include "sg_internal.cuh"
#include "sg_asm_api.h"

namespace sg {
namespace SG_ASM_NS {

template <class Elem, int G, int BS, typename T>
static int launch_rows(Ctx *c, AsmArgs<T> &a) {
  if (a.n == 0) return SG_OK;
  const int maxrow = Elem::HAS_MAT ? a.maxrow : 0;
  const size_t per_group = (size_t)maxrow * (BS * BS * sizeof(T) + 4);
  int threads = 128;
  while (threads > G && (threads / G) * per_group > 96 * 1024) threads >>= 1;
  if ((threads / G) * per_group > 96 * 1024)
    return set_error(SG_ERR_UNSUPPORTED, "assembly: a row of %d blocks exceeds shared memory",
                     maxrow);
  const size_t sh = (threads / G) * per_group;
  if (sh > 48 * 1024)
    SG_CHECK_CUDA(cudaFuncSetAttribute(k_rows<Elem, G, BS, T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh));
  a.err = c->d_err;
  const int grid = grid_for(c, (int64_t)a.n * G, threads, 16);
  k_rows<Elem, G, BS, T><<<grid, threads, sh, c->stream>>>(a);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// The element-parallel form over the mesh's colouring plan (fast
// instantiation only; the exact one keeps the reference's element order
// through the row owners).  Outputs are zeroed first, then one launch per
// colour.  Returns 1 through *used when it ran.
template <class Elem, int CARD, int BS, typename T>
static int launch_colored(Ctx *c, AsmArgs<T> &a, const sg_mesh *m, bool *used) {
  *used = false;
  if (SG_ASM_EXACT || !m->slots || m->card != CARD) return SG_OK;
  a.err = c->d_err;
  if (m->slot_src_ptr && m->slot_src) {
    // element blocks (context scratch) + slot / vertex gathers
    constexpr bool SY = elem_sym<Elem>::value;
    constexpr int BPE = SY ? CARD * (CARD + 1) / 2 : CARD * CARD;  // stored blocks per element
    const size_t neb = Elem::HAS_MAT ? (size_t)m->nE * BPE * BS * BS : 0;
    const size_t nev = Elem::HAS_VEC ? (size_t)m->nE * CARD * BS : 0;
    Scratch s(c);
    SG_TRY(s.reserve(Scratch::bytes_for(neb + 1, sizeof(T)) + Scratch::bytes_for(nev + 1, sizeof(T))));
    T *eb = s.alloc<T>(neb + 1), *ev = s.alloc<T>(nev + 1);
    if (m->nE > 0) {
      const int64_t th = m->nE * (Elem::HAS_MAT ? BPE : CARD);
      const int tile = m->asm_tile;
      if (tile == 128)
        k_elem_blocks<Elem, CARD, BS, T, 128><<<grid_for(c, th, 128, 16), 128, 0, c->stream>>>(
            a, eb, ev);
      else if (tile == 512)
        k_elem_blocks<Elem, CARD, BS, T, 512><<<grid_for(c, th, 512, 4), 512, 0, c->stream>>>(
            a, eb, ev);
      else
        k_elem_blocks<Elem, CARD, BS, T, 256><<<grid_for(c, th, 256, 8), 256, 0, c->stream>>>(
            a, eb, ev);
      SG_CHECK_LAUNCH();
    }
    if (Elem::HAS_MAT && m->nnzb > 0) {
      k_slot_gather<BS, T, SY ? CARD : 0><<<grid_for(c, m->nnzb * BS, 256, 8), 256, 0, c->stream>>>(
          m->nnzb, m->slot_src_ptr, m->slot_src, eb, a.vals);
      SG_CHECK_LAUNCH();
    }
    if (Elem::HAS_VEC && m->n > 0) {
      k_vert_gather<BS, T><<<grid_for(c, (int64_t)m->n * BS, 256, 8), 256, 0, c->stream>>>(
          m->n, m->ve_ptr, m->ve_idx, ev, a.f);
      SG_CHECK_LAUNCH();
    }
    *used = true;
    return SG_OK;
  }
  if (!m->color_order || !m->color_ptr || m->ncolors <= 0) return SG_OK;
  if (Elem::HAS_MAT)
    SG_CHECK_CUDA(cudaMemsetAsync(a.vals, 0, (size_t)m->nnzb * BS * BS * sizeof(T), c->stream));
  if (Elem::HAS_VEC)
    SG_CHECK_CUDA(cudaMemsetAsync(a.f, 0, (size_t)m->n * BS * sizeof(T), c->stream));
  for (int k = 0; k < m->ncolors; ++k) {
    const int64_t b0 = m->color_ptr[k], cnt = (int64_t)m->color_ptr[k + 1] - b0;
    if (cnt <= 0) continue;
    const int64_t threads = cnt * (Elem::HAS_MAT ? CARD * CARD : CARD);
    k_colored<Elem, CARD, BS, T><<<grid_for(c, threads, 256, 8), 256, 0, c->stream>>>(
        a, m->color_order + b0, cnt, m->slots);
    SG_CHECK_LAUNCH();
  }
  *used = true;
  return SG_OK;
}

template <typename T>
static void fill_mesh(AsmArgs<T> &a, const sg_mesh *m) {
  a.n = m->n;
  a.card = m->card;
  a.nE = m->nE;
  a.ep = m->endpoints;
  a.ve_ptr = m->ve_ptr;
  a.ve_idx = m->ve_idx;
  a.rowptr = m->rowptr;
  a.colidx = m->colidx;
  a.maxrow = m->maxrow;
  a.nnzb = m->nnzb;
}

template <typename T>
int springs(Ctx *c, const sg_mesh *m, int form, const void *x, const void *v, const void *mass,
            const uint8_t *fixed, const void *k, const void *l0, double h, double viscous,
            const double *grav, void *vals, void *f) {
  AsmArgs<T> a;
  fill_mesh(a, m);
  a.x = (const T *)x; a.v = (const T *)v; a.m = (const T *)mass; a.fixed = fixed;
  a.k = (const T *)k; a.l0 = (const T *)l0; a.h = (T)h; a.viscous = (T)viscous;
  for (int q = 0; q < 3; ++q) a.grav[q] = (T)grav[q];
  a.form = form;
  a.vals = (T *)vals; a.f = (T *)f;
  return launch_rows<SpringElem<T>, 8, 3, T>(c, a);
}

template <typename T>
int scalar_springs(Ctx *c, const sg_mesh *m, const void *av, double diag, double scale,
                   void *vals) {
  AsmArgs<T> a;
  fill_mesh(a, m);
  a.a = (const T *)av; a.diag = (T)diag; a.scale = (T)scale; a.vals = (T *)vals;
  return launch_rows<ScalarSpringElem<T>, 2, 1, T>(c, a);
}

template <typename T>
int heat(Ctx *c, const sg_mesh *m, const void *B, const void *W, const void *kappa, double dt,
         const void *T0, void *vals, void *b) {
  AsmArgs<T> a;
  fill_mesh(a, m);
  a.B = (const T *)B; a.W = (const T *)W; a.kappa = (const T *)kappa; a.dt = (T)dt;
  a.T0 = (const T *)T0; a.vals = (T *)vals; a.f = (T *)b;
  bool used = false;
  SG_TRY((launch_colored<HeatElem<T>, 4, 1, T>(c, a, m, &used)));
  if (used) return SG_OK;
  return launch_rows<HeatElem<T>, 4, 1, T>(c, a);
}

template <typename T>
int tet_precompute(Ctx *c, const sg_mesh *m, const void *x, double rho, void *B, void *W,
                   void *mass) {
  if (m->nE > 0) {
    k_tet_precompute<T><<<grid_for(c, m->nE, 128, 16), 128, 0, c->stream>>>(
        m->nE, m->endpoints, (const T *)x, (T *)B, (T *)W);
    SG_CHECK_LAUNCH();
  }
  AsmArgs<T> a;
  fill_mesh(a, m);
  a.W = (const T *)W; a.rho = (T)rho; a.f = (T *)mass;
  return launch_rows<TetMassElem<T>, 1, 1, T>(c, a);
}

template <typename T>
int blocks(Ctx *c, const sg_mesh *m, int bs, const void *eb, void *vals) {
  AsmArgs<T> a;
  fill_mesh(a, m);
  a.eb = (const T *)eb;
  a.vals = (T *)vals;
#define SG_BLK(BSV, CV)                                                            \
  if (bs == BSV && m->card == CV) {                                                \
    bool used = false;                                                             \
    SG_TRY((launch_colored<BlocksElem<T, BSV, CV>, CV, BSV, T>(c, a, m, &used)));  \
    if (used) return SG_OK;                                                        \
    return launch_rows<BlocksElem<T, BSV, CV>, 16, BSV, T>(c, a);                  \
  }
  SG_BLK(1, 2) SG_BLK(1, 3) SG_BLK(1, 4)
  SG_BLK(2, 2) SG_BLK(2, 3) SG_BLK(2, 4)
  SG_BLK(3, 2) SG_BLK(3, 3) SG_BLK(3, 4)
#undef SG_BLK
  return set_error(SG_ERR_UNSUPPORTED, "sg_assemble_blocks: bs %d, card %d (bs 1..3, card 2..4)",
                   bs, m->card);
}

template <typename T>
int tet_stiffness(Ctx *c, const sg_mesh *m, int model, const void *x, const int32_t *cons,
                  const void *B, const void *W, const void *mu, const void *lam, double h,
                  double rho, void *vals, void *eb_scratch) {
  AsmArgs<T> a;
  fill_mesh(a, m);
  a.x = (const T *)x; a.c = cons; a.B = (const T *)B; a.W = (const T *)W;
  a.mu = (const T *)mu; a.lam = (const T *)lam; a.h = (T)h; a.rho = (T)rho;
  a.vals = (T *)vals;
  if (model == SG_MODEL_NEOHOOKEAN) {
    a.eb = (const T *)eb_scratch;
    if (m->nE > 0) {
      k_neo_blocks<T><<<grid_for(c, m->nE, 128, 16), 128, 0, c->stream>>>(a);
      SG_CHECK_LAUNCH();
    }
    bool used = false;
    SG_TRY((launch_colored<EbGatherElem<T>, 4, 3, T>(c, a, m, &used)));
    if (used) return SG_OK;
    return launch_rows<EbGatherElem<T>, 16, 3, T>(c, a);
  }
  bool used = false;
  SG_TRY((launch_colored<LinTetElem<T, SG_ASM_EXACT>, 4, 3, T>(c, a, m, &used)));
  if (used) return SG_OK;
  return launch_rows<LinTetElem<T, SG_ASM_EXACT>, 16, 3, T>(c, a);
}

template <typename T>
int tet_force(Ctx *c, const sg_mesh *m, int model, const void *x, const void *v,
              const int32_t *cons, const void *B, const void *W, const void *mu, const void *lam,
              double h, double rho, const double *grav, void *f) {
  AsmArgs<T> a;
  fill_mesh(a, m);
  a.x = (const T *)x; a.v = (const T *)v; a.c = cons; a.B = (const T *)B; a.W = (const T *)W;
  a.mu = (const T *)mu; a.lam = (const T *)lam; a.h = (T)h; a.rho = (T)rho;
  for (int q = 0; q < 3; ++q) a.grav[q] = (T)grav[q];
  a.f = (T *)f;
  bool used = false;
  if (model == SG_MODEL_NEOHOOKEAN) {
    SG_TRY((launch_colored<TetForceElem<T, true>, 4, 3, T>(c, a, m, &used)));
    if (used) return SG_OK;
    return launch_rows<TetForceElem<T, true>, 4, 3, T>(c, a);
  }
  SG_TRY((launch_colored<TetForceElem<T, false>, 4, 3, T>(c, a, m, &used)));
  if (used) return SG_OK;
  return launch_rows<TetForceElem<T, false>, 4, 3, T>(c, a);
}

// Explicit instantiations for both precisions.
#define SG_INST(T)                                                                        \
  template int springs<T>(Ctx *, const sg_mesh *, int, const void *, const void *,       \
                          const void *, const uint8_t *, const void *, const void *, double, \
                          double, const double *, void *, void *);                       \
  template int scalar_springs<T>(Ctx *, const sg_mesh *, const void *, double, double,    \
                                 void *);                                                 \
  template int heat<T>(Ctx *, const sg_mesh *, const void *, const void *, const void *,   \
                       double, const void *, void *, void *);                             \
  template int tet_precompute<T>(Ctx *, const sg_mesh *, const void *, double, void *,    \
                                 void *, void *);                                         \
  template int blocks<T>(Ctx *, const sg_mesh *, int, const void *, void *);               \
  template int tet_stiffness<T>(Ctx *, const sg_mesh *, int, const void *, const int32_t *, \
                                const void *, const void *, const void *, const void *,   \
                                double, double, void *, void *);                          \
  template int tet_force<T>(Ctx *, const sg_mesh *, int, const void *, const void *,      \
                            const int32_t *, const void *, const void *, const void *,    \
                            const void *, double, double, const double *, void *);
SG_INST(float)
SG_INST(double)
#undef SG_INST

}  // namespace SG_ASM_NS
}  // namespace sg
