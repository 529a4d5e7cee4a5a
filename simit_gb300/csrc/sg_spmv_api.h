// Internal launch helpers of the SpMV kernels (used by sg_bspmv and the CG).
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace sg {
struct Ctx;
struct PatternStats {
  int maxrow = 0, tile16 = 0, tile32 = 0, tile4 = 0, tile8 = 0;
};
int default_lanes(int32_t n, int64_t nnzb, int32_t bs);
int default_tma_variant(int bs);
int cached_maxrow(Ctx *c, int32_t n, const uint32_t *rowptr, int *out);
int cached_stats(Ctx *c, int32_t n, const uint32_t *rowptr, PatternStats *ps,
                 bool refresh = false);
int bspmv_launch(Ctx *c, int32_t n, int32_t bs, const uint32_t *rp, const uint32_t *ci, int vdt,
                 const void *v, int xdt, const void *x, void *y, int g, int64_t nnzb_hint);
// TMA-staged SpMV (bs = 3: every variant; bs = 1: the per-warp variants):
// grid/shared-memory for variant `var` (see kTmaVariants in sg_spmv.cu);
// launch.  dot = 1 also writes per-CTA partials of x.y (CG K1) and honours
// ctl.  SG_ERR_UNSUPPORTED when the variant cannot run this pattern.
int bsr3_tma_config(Ctx *c, int bs, int vdt, int xdt, int var, int dot, int32_t n,
                    const PatternStats &ps, int *grid, size_t *smem);
int bsr3_tma_launch(Ctx *c, cudaStream_t st, const void *ctl, int bs, int vdt, int xdt, int var,
                    int dot, int32_t n, const uint32_t *rp, const uint32_t *ci, const void *v,
                    const void *x, void *y, double *part, const PatternStats &ps, int grid,
                    size_t smem);
}  // namespace sg
