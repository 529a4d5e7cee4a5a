// Declarations of the assembly launchers instantiated in sg_assemble_exact.cu
// (namespace sg::exact, --fmad=false, reference operation order) and
// sg_assemble_fast.cu (namespace sg::fast).
#pragma once
#include <stdint.h>

#include "../../include/simit_gb300.h"

namespace sg {
struct Ctx;
#define SG_ASM_DECL(NS)                                                                   \
  namespace NS {                                                                          \
  template <typename T>                                                                   \
  int springs(Ctx *, const sg_mesh *, int, const void *, const void *, const void *,     \
              const uint8_t *, const void *, const void *, double, double, const double *, \
              void *, void *);                                                            \
  template <typename T>                                                                   \
  int scalar_springs(Ctx *, const sg_mesh *, const void *, double, double, void *);       \
  template <typename T>                                                                   \
  int heat(Ctx *, const sg_mesh *, const void *, const void *, const void *, double,      \
           const void *, void *, void *);                                                 \
  template <typename T>                                                                   \
  int tet_precompute(Ctx *, const sg_mesh *, const void *, double, void *, void *, void *); \
  template <typename T>                                                                   \
  int blocks(Ctx *, const sg_mesh *, int, const void *, void *);                          \
  template <typename T>                                                                   \
  int tet_stiffness(Ctx *, const sg_mesh *, int, const void *, const int32_t *,           \
                    const void *, const void *, const void *, const void *, double, double, \
                    void *, void *);                                                      \
  template <typename T>                                                                   \
  int tet_force(Ctx *, const sg_mesh *, int, const void *, const void *, const int32_t *, \
                const void *, const void *, const void *, const void *, double, double,   \
                const double *, void *);                                                  \
  }
SG_ASM_DECL(exact)
SG_ASM_DECL(fast)
#undef SG_ASM_DECL
}  // namespace sg
