/* simit_gb300 — C ABI of the GB300 sparse-system path (assembly over edge
 * sets into blocked CSR, blocked SpMV, conjugate-gradient solves).
 *
 * Conventions
 *   - Every entry point returns int: SG_OK (0) or a negative SG_ERR_* code; it
 *     never throws.  sg_last_error() gives a message for the calling thread.
 *     The C++ facade (simit_gb300/cpp/simit.h) turns a negative code into an
 *     exception, as the reference's simit_uassert raises SimitException
 *     (src/error.cpp:86-97).
 *   - Array arguments are DEVICE pointers unless the name starts with h_.
 *     Sizes are element counts.  Nothing here takes torch types.
 *   - Calls are asynchronous on the context's stream unless documented as
 *     synchronising (those that return a size or a solver result).
 *   - A context is not thread-safe; use one per host thread.
 *   - Blocked CSR layout is the reference's Indexed storage
 *     (src/lower/lower_accesses.cpp:120-245): rowptr uint32[n+1],
 *     colidx uint32[nnzb] sorted ascending within each row, values
 *     T[nnzb * bs * bs], each block row-major.
 *   - Element endpoints are the reference's edge-set layout
 *     int32[nE * card] row-major (src/graph.h:429-431, 621).
 */
#ifndef SIMIT_GB300_H
#define SIMIT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SG_OK = 0,
  SG_ERR_ARG = -1,          /* bad argument (null, size, dtype, ...) */
  SG_ERR_CUDA = -2,         /* CUDA runtime error */
  SG_ERR_UNSUPPORTED = -3,  /* valid input outside what a kernel supports */
  SG_ERR_DEVICE = -4,       /* a device-side check failed (bad index, ...) */
  SG_ERR_STATE = -5         /* wrong call order / handle state */
};

enum { SG_F32 = 0, SG_F64 = 1 };

typedef struct sg_ctx sg_ctx;

/* Context: binds a device and creates one stream.
 * Replaces the device set-up of GPUFunction::init
 * (src/backend/gpu/gpu_function.cpp:113-138, 180-560). */
int sg_ctx_create(int device, sg_ctx **out);
int sg_ctx_destroy(sg_ctx *ctx);
int sg_ctx_sync(sg_ctx *ctx);
/* The context's stream as an opaque pointer (a cudaStream_t). */
void *sg_ctx_stream(sg_ctx *ctx);
const char *sg_last_error(void);
const char *sg_version(void);

/* ---------------------------------------------------------------------
 * Pattern construction.  Replaces pe::PathIndexBuilder::buildSegmented for
 * the assembly expression ∃e∈E.(v-e ∧ e-u) (src/path_indices.cpp:148-531,
 * built per src/path_expression_analysis.cpp:84-91) and the per-element
 * `loc` slot searches (src/runtime.cpp:19-23, src/inline.cpp:524-577).
 * Results are bit-identical to the reference's.
 * ------------------------------------------------------------------- */

/* Vertex -> (element*card + i) incidence, rows sorted ascending (the
 * reference's Link::ve index, src/path_indices.cpp:248-276, extended with the
 * endpoint position).  ve_ptr uint32[n+1], ve_idx uint32[nE*card]. */
int sg_incidence_build(sg_ctx *ctx, int32_t n, const int32_t *endpoints,
                       int64_t nE, int32_t card, uint32_t *ve_ptr,
                       uint32_t *ve_idx);

/* Row pointers of the pattern; synchronises and returns nnzb. */
int sg_pattern_count(sg_ctx *ctx, int32_t n, const int32_t *endpoints,
                     int64_t nE, int32_t card, const uint32_t *ve_ptr,
                     const uint32_t *ve_idx, uint32_t *rowptr,
                     int64_t *h_nnzb);

/* Column indices (sorted, unique per row) after sg_pattern_count. */
int sg_pattern_fill(sg_ctx *ctx, int32_t n, const int32_t *endpoints,
                    int64_t nE, int32_t card, const uint32_t *ve_ptr,
                    const uint32_t *ve_idx, const uint32_t *rowptr,
                    uint32_t *colidx);

/* Element-to-slot map slots[(e*card + i)*card + j] = slot of block
 * (ep[e,i], ep[e,j]) — the reference's `.K_index_locs`. */
int sg_slots_build(sg_ctx *ctx, int32_t n, const int32_t *endpoints,
                   int64_t nE, int32_t card, const uint32_t *rowptr,
                   const uint32_t *colidx, uint32_t *slots);

/* ---------------------------------------------------------------------
 * Blocked SpMV  y = A x.  Replaces the lowered SpMV loop nest
 * (src/lower/index_expressions/lower_indexexprs.cpp:630-660).
 * bs = 1, 2, 3 have dedicated kernels; other bs use a generic kernel.
 * val_dtype is the matrix value type; vec_dtype the type of x and y;
 * accumulation is in the wider of the two.  g = lanes per block row
 * (0 = autotuned choice; else 1,2,4,8,16,32).
 * ------------------------------------------------------------------- */
int sg_bspmv(sg_ctx *ctx, int32_t n, int32_t bs, const uint32_t *rowptr,
             const uint32_t *colidx, int val_dtype, const void *vals,
             int vec_dtype, const void *x, void *y, int32_t g);

/* Dot product of two blocked vectors with an FP64 deterministic two-level
 * reduction; synchronises. */
int sg_dot(sg_ctx *ctx, int64_t len, int vec_dtype, const void *a,
           const void *b, double *h_out);

#ifdef __cplusplus
}
#endif
#endif /* SIMIT_GB300_H */
