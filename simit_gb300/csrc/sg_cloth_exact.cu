// Cloth forces of the reference's cloth example (apps/cloth/cloth.sim):
// triangle stretching over faces (card 3, stretchingForce, :142-164) and
// dihedral bending over hinges (card 4, bendingForce, :166-173), assembled
// into a system vector (`map ... reduce +`).  A thread owns a vertex and
// adds, from zero, its incidences' terms in ascending (element, local
// index), each element's terms in the program's order -- the order of the
// lowered map's `+=`, so FP64 sums equal the reference's.  Compiled with
// --fmad=false (a *_exact.cu unit): no multiply-add contraction.
#include "sg_internal.cuh"

namespace sg {
namespace {

template <typename T> __device__ __forceinline__ T dot3(const T *a, const T *b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}
template <typename T> __device__ __forceinline__ void cross3(const T *a, const T *b, T *r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
template <typename T> __device__ __forceinline__ void sub3(const T *a, const T *b, T *r) {
  for (int q = 0; q < 3; ++q) r[q] = a[q] - b[q];
}
template <typename T> __device__ __forceinline__ void load3(const T *x, int32_t v, T *o) {
  for (int q = 0; q < 3; ++q) o[q] = x[(int64_t)v * 3 + q];
}

// The dihedral angle at edge p1-p2 between triangles (p1, p2, q1) and
// (p1, p2, q2) (cloth.sim:31-38, computeAngle).
template <typename T>
__device__ T cloth_angle(const T *p1, const T *p2, const T *q1, const T *q2) {
  T ev[3], d1[3], d2[3], n1[3], n2[3], c[3];
  sub3(p2, p1, ev);
  sub3(q1, p1, d1);
  cross3(ev, d1, n1);
  sub3(q2, p1, d2);
  cross3(d2, ev, n2);
  const T mag = sqrt(dot3(ev, ev));
  for (int q = 0; q < 3; ++q) ev[q] = ev[q] / mag;
  cross3(n1, n2, c);
  return atan2(dot3(c, ev), dot3(n1, n2));
}

// d theta / d vertex a of the hinge (cloth.sim:115-140,
// dihedralAngleDerivatives).
template <typename T>
__device__ void cloth_angle_grad(const T *p1, const T *p2, const T *q1, const T *q2, int a,
                                 T *g) {
  T v11[3], v12[3], v21[3], v22[3], v[3], n1[3], n2[3];
  sub3(q1, p2, v11);
  sub3(q1, p1, v12);
  sub3(q2, p2, v21);
  sub3(q2, p1, v22);
  sub3(p2, p1, v);
  cross3(v12, v, n1);
  cross3(v, v22, n2);
  const T n1n2 = dot3(n1, n1), n2n2 = dot3(n2, n2), vn = sqrt(dot3(v, v));
  if (vn < T(1e-8) || n1n2 < T(1e-8) || n2n2 < T(1e-8)) {
    g[0] = g[1] = g[2] = T(0);
    return;
  }
  T m12[3], m22[3];
  for (int q = 0; q < 3; ++q) {
    m12[q] = -v12[q];
    m22[q] = -v22[q];
  }
  const T a11 = dot3(v11, v), a21 = dot3(v21, v), a12 = dot3(m12, v), a22 = dot3(m22, v);
  for (int q = 0; q < 3; ++q) {
    if (a == 2) g[q] = (n1[q] * vn) / n1n2;
    else if (a == 3) g[q] = (n2[q] * vn) / n2n2;
    else if (a == 0) g[q] = ((n1[q] * a11) / vn) / n1n2 + ((n2[q] * a21) / vn) / n2n2;
    else g[q] = ((n1[q] * a12) / vn) / n1n2 + ((n2[q] * a22) / vn) / n2n2;
  }
}

template <typename T>
__global__ void __launch_bounds__(128)
    k_cloth_stretch(int32_t n, const uint32_t *__restrict__ ve_ptr,
                    const uint32_t *__restrict__ ve_idx, const int32_t *__restrict__ ep,
                    const T *__restrict__ x, const T *__restrict__ K, const T *__restrict__ rest,
                    T *__restrict__ f) {
  for (int64_t vtx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vtx < n;
       vtx += (int64_t)gridDim.x * blockDim.x) {
    T acc[3] = {T(0), T(0), T(0)};
    for (uint32_t it = ve_ptr[vtx]; it < ve_ptr[vtx + 1]; ++it) {
      const uint32_t t = ve_idx[it];
      const int64_t e = t / 3;
      const int k = (int)(t - (uint32_t)e * 3);
      T p0[3], p1[3], p2[3], v[3][3];
      load3(x, ep[e * 3], p0);
      load3(x, ep[e * 3 + 1], p1);
      load3(x, ep[e * 3 + 2], p2);
      // v_c: the current edge opposite corner c; s_i: its squared length
      // less the rest one (rest lengths are stored for edges 01, 12, 20)
      sub3(p2, p1, v[0]);
      sub3(p0, p2, v[1]);
      sub3(p1, p0, v[2]);
      const T r[3] = {rest[e * 3 + 1], rest[e * 3 + 2], rest[e * 3]};
      T s[3];
      for (int i = 0; i < 3; ++i) s[i] = dot3(v[i], v[i]) - r[i];
      const T *Ke = K + e * 9;
      const int k2 = (k + 1) % 3, k1 = (k + 2) % 3;
      for (int i = 0; i < 3; ++i)
        for (int q = 0; q < 3; ++q) {
          const T tt = (Ke[i * 3 + k2] * s[i]) * v[k2][q] - (Ke[i * 3 + k1] * s[i]) * v[k1][q];
          acc[q] += T(-4.0) * tt;
        }
    }
    for (int q = 0; q < 3; ++q) f[vtx * 3 + q] = acc[q];
  }
}

template <typename T>
__global__ void __launch_bounds__(128)
    k_cloth_bend(int32_t n, const uint32_t *__restrict__ ve_ptr,
                 const uint32_t *__restrict__ ve_idx, const int32_t *__restrict__ ep,
                 const T *__restrict__ x, const T *__restrict__ angle, const T *__restrict__ len,
                 const T *__restrict__ perp, T *__restrict__ f) {
  for (int64_t vtx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; vtx < n;
       vtx += (int64_t)gridDim.x * blockDim.x) {
    T acc[3] = {T(0), T(0), T(0)};
    for (uint32_t it = ve_ptr[vtx]; it < ve_ptr[vtx + 1]; ++it) {
      const uint32_t t = ve_idx[it];
      const int64_t h = t / 4;
      const int a = (int)(t - (uint32_t)h * 4);
      T p[4][3];
      for (int j = 0; j < 4; ++j) load3(x, ep[h * 4 + j], p[j]);
      const T dth = cloth_angle(p[0], p[1], p[2], p[3]) - angle[h];
      T g[3];
      cloth_angle_grad(p[0], p[1], p[2], p[3], a, g);
      for (int q = 0; q < 3; ++q) acc[q] += (((-g[q]) * len[h]) / perp[h]) * dth;
    }
    for (int q = 0; q < 3; ++q) f[vtx * 3 + q] = acc[q];
  }
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" {

int sg_assemble_cloth_stretch(sg_ctx *h, const sg_mesh *m, int dtype, const void *x,
                              const void *K, const void *rest, void *f) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && m && x && K && rest && f, "sg_assemble_cloth_stretch: null argument");
  SG_REQUIRE(m->card == 3, "sg_assemble_cloth_stretch: faces have 3 endpoints, not %d", m->card);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_assemble_cloth_stretch: dtype %d", dtype);
  SG_REQUIRE(m->ve_ptr && (m->nE == 0 || (m->ve_idx && m->endpoints)),
             "sg_assemble_cloth_stretch: mesh incidence missing");
  if (m->n == 0) return SG_OK;
  const int G = grid_for(c, m->n, 128, 8);
  if (dtype == SG_F64)
    k_cloth_stretch<double><<<G, 128, 0, c->stream>>>(m->n, m->ve_ptr, m->ve_idx, m->endpoints,
                                                      (const double *)x, (const double *)K,
                                                      (const double *)rest, (double *)f);
  else
    k_cloth_stretch<float><<<G, 128, 0, c->stream>>>(m->n, m->ve_ptr, m->ve_idx, m->endpoints,
                                                     (const float *)x, (const float *)K,
                                                     (const float *)rest, (float *)f);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

int sg_assemble_cloth_bend(sg_ctx *h, const sg_mesh *m, int dtype, const void *x,
                           const void *angle, const void *len, const void *perp, void *f) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && m && x && angle && len && perp && f, "sg_assemble_cloth_bend: null argument");
  SG_REQUIRE(m->card == 4, "sg_assemble_cloth_bend: hinges have 4 endpoints, not %d", m->card);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_assemble_cloth_bend: dtype %d", dtype);
  SG_REQUIRE(m->ve_ptr && (m->nE == 0 || (m->ve_idx && m->endpoints)),
             "sg_assemble_cloth_bend: mesh incidence missing");
  if (m->n == 0) return SG_OK;
  const int G = grid_for(c, m->n, 128, 8);
  if (dtype == SG_F64)
    k_cloth_bend<double><<<G, 128, 0, c->stream>>>(m->n, m->ve_ptr, m->ve_idx, m->endpoints,
                                                   (const double *)x, (const double *)angle,
                                                   (const double *)len, (const double *)perp,
                                                   (double *)f);
  else
    k_cloth_bend<float><<<G, 128, 0, c->stream>>>(m->n, m->ve_ptr, m->ve_idx, m->endpoints,
                                                  (const float *)x, (const float *)angle,
                                                  (const float *)len, (const float *)perp,
                                                  (float *)f);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // extern "C"
