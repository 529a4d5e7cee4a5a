// C ABI of the assembly kernels: argument checks and exact/fast dispatch.
#include "sg_asm_api.h"
#include "sg_internal.cuh"

namespace sg {
__global__ void max_u32_diff(const uint32_t *ptr, int32_t n, uint32_t *out);

static int check_mesh(const sg_mesh *m, bool need_pattern, const char *who) {
  SG_REQUIRE(m, "%s: mesh is null", who);
  SG_REQUIRE(m->n >= 0 && m->nE >= 0 && m->card >= 1, "%s: bad mesh sizes", who);
  SG_REQUIRE(m->ve_ptr && (m->nE == 0 || (m->endpoints && m->ve_idx)),
             "%s: mesh incidence missing", who);
  if (need_pattern) {
    SG_REQUIRE(m->rowptr && (m->nnzb == 0 || m->colidx), "%s: mesh pattern missing", who);
    SG_REQUIRE(m->maxrow >= 0 && m->maxrow <= 4096, "%s: maxrow %d out of range", who,
               m->maxrow);
  }
  return SG_OK;
}
}  // namespace sg

using namespace sg;

#define SG_DISPATCH(EX, dtype, FN, ...)                                        \
  ((EX) ? ((dtype) == SG_F64 ? exact::FN<double>(__VA_ARGS__)             \
                                : exact::FN<float>(__VA_ARGS__))              \
           : ((dtype) == SG_F64 ? fast::FN<double>(__VA_ARGS__)              \
                                : fast::FN<float>(__VA_ARGS__)))

extern "C" {

int sg_pattern_maxrow(sg_ctx *h, int32_t n, const uint32_t *rowptr, int32_t *h_maxrow) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && rowptr && h_maxrow, "sg_pattern_maxrow: null argument");
  if (n <= 0) {
    *h_maxrow = 0;
    return SG_OK;
  }
  Scratch s(c);
  SG_TRY(s.reserve(256));
  uint32_t *d = s.alloc<uint32_t>(1);
  SG_CHECK_CUDA(cudaMemsetAsync(d, 0, 4, c->stream));
  max_u32_diff<<<grid_for(c, n, 256, 4), 256, 0, c->stream>>>(rowptr, n, d);
  SG_CHECK_LAUNCH();
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, d, 4, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  *h_maxrow = (int32_t) * (uint32_t *)c->h_stage;
  return SG_OK;
}

int sg_assemble_springs(sg_ctx *h, const sg_mesh *m, int dt, int form, const void *x,
                        const void *v, const void *mass, const uint8_t *fixed, const void *k,
                        const void *l0, double hh, double viscous, const double *grav,
                        void *vals, void *f, int exact) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_assemble_springs: null context");
  SG_TRY(check_mesh(m, true, "sg_assemble_springs"));
  SG_REQUIRE(m->card == 2, "sg_assemble_springs: springs have 2 endpoints, got %d", m->card);
  SG_REQUIRE(x && v && mass && fixed && grav && vals && f && (m->nE == 0 || (k && l0)),
             "sg_assemble_springs: null array");
  SG_REQUIRE(form == 0 || form == 1, "sg_assemble_springs: form %d", form);
  SG_TRY(SG_DISPATCH(exact, dt, springs, c, m, form, x, v, mass, fixed, k, l0, hh, viscous,
                     grav, vals, f));
  return SG_OK;
}

int sg_assemble_scalar_springs(sg_ctx *h, const sg_mesh *m, int dt, const void *a,
                               double diag, double scale, void *vals, int exact) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_assemble_scalar_springs: null context");
  SG_TRY(check_mesh(m, true, "sg_assemble_scalar_springs"));
  SG_REQUIRE(m->card == 2 && vals && (m->nE == 0 || a), "sg_assemble_scalar_springs: bad args");
  return SG_DISPATCH(exact, dt, scalar_springs, c, m, a, diag, scale, vals);
}

int sg_assemble_blocks(sg_ctx *h, const sg_mesh *m, int dt, int bs, const void *eb, void *vals,
                       int exact) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_assemble_blocks: null context");
  SG_TRY(check_mesh(m, true, "sg_assemble_blocks"));
  SG_REQUIRE(bs >= 1 && bs <= 3 && m->card >= 2 && m->card <= 4,
             "sg_assemble_blocks: bs %d card %d (bs 1..3, card 2..4)", bs, m->card);
  SG_REQUIRE(vals && (m->nE == 0 || eb), "sg_assemble_blocks: null array");
  return SG_DISPATCH(exact, dt, blocks, c, m, bs, eb, vals);
}

int sg_tet_precompute(sg_ctx *h, const sg_mesh *m, int dt, const void *x, double rho, void *B,
                      void *W, void *mass) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_tet_precompute: null context");
  SG_TRY(check_mesh(m, false, "sg_tet_precompute"));
  SG_REQUIRE(m->card == 4 && x && mass && (m->nE == 0 || (B && W)),
             "sg_tet_precompute: bad args");
  return SG_DISPATCH(1, dt, tet_precompute, c, m, x, rho, B, W, mass);
}

int sg_assemble_tet_stiffness(sg_ctx *h, const sg_mesh *m, int dt, int model, const void *x,
                              const int32_t *cons, const void *B, const void *W, const void *mu,
                              const void *lam, double hh, double rho, void *vals, int exact) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_assemble_tet_stiffness: null context");
  SG_TRY(check_mesh(m, true, "sg_assemble_tet_stiffness"));
  SG_REQUIRE(m->card == 4 && cons && vals && (m->nE == 0 || (B && W && mu && lam)),
             "sg_assemble_tet_stiffness: bad args");
  SG_REQUIRE(model == SG_MODEL_LINEAR || model == SG_MODEL_NEOHOOKEAN,
             "sg_assemble_tet_stiffness: model %d", model);
  SG_REQUIRE(model == SG_MODEL_LINEAR || x, "sg_assemble_tet_stiffness: x is null");
  void *eb = nullptr;
  Scratch s(c);
  if (model == SG_MODEL_NEOHOOKEAN) {
    const size_t bytes = (size_t)m->nE * 144 * dtype_size(dt);
    SG_TRY(s.reserve(bytes + 256));
    eb = s.alloc<char>(bytes);
  }
  return SG_DISPATCH(exact, dt, tet_stiffness, c, m, model, x, cons, B, W, mu, lam, hh, rho,
                     vals, eb);
}

int sg_assemble_tet_force(sg_ctx *h, const sg_mesh *m, int dt, int model, const void *x,
                          const void *v, const int32_t *cons, const void *B, const void *W,
                          const void *mu, const void *lam, double hh, double rho,
                          const double *grav, void *f, int exact) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_assemble_tet_force: null context");
  SG_TRY(check_mesh(m, false, "sg_assemble_tet_force"));
  SG_REQUIRE(m->card == 4 && x && v && cons && grav && f && (m->nE == 0 || (B && W && mu && lam)),
             "sg_assemble_tet_force: bad args");
  return SG_DISPATCH(exact, dt, tet_force, c, m, model, x, v, cons, B, W, mu, lam, hh, rho, grav,
                     f);
}

int sg_assemble_heat(sg_ctx *h, const sg_mesh *m, int dt, const void *B, const void *W,
                     const void *kappa, double dtt, const void *T0, void *vals, void *b,
                     int exact) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c, "sg_assemble_heat: null context");
  SG_TRY(check_mesh(m, true, "sg_assemble_heat"));
  SG_REQUIRE(m->card == 4 && T0 && vals && b && (m->nE == 0 || (B && W && kappa)),
             "sg_assemble_heat: bad args");
  return SG_DISPATCH(exact, dt, heat, c, m, B, W, kappa, dtt, T0, vals, b);
}

}  // extern "C"
