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
/* Releases the caller's reference; the context (and its stream) lives on
 * until every solver created on it has been destroyed too. */
int sg_ctx_destroy(sg_ctx *ctx);
/* Waits for the context's stream, then reports (SG_ERR_DEVICE) and clears a
 * device-side check that failed in an asynchronous call since the last
 * check (an assembly row longer than its bound, a missing diagonal block). */
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

/* Incidence matrices of an edge set over one of its vertex sets, the
 * reference's non-square assembly patterns (src/path_expression_analysis
 * .cpp:95-105).  sel int32[nE*npos]: each element's endpoints that lie in
 * that vertex set, in endpoint order (all card endpoints for a homogeneous
 * edge set); n: that vertex set's size.
 *   SG_INCIDENCE_EV, tensor[E,V] (Link::ev, src/path_indices.cpp:207-246):
 *     rowptr[nE+1] = e*npos, colidx[nE*npos] = sel (repeats kept);
 *     slot_of unused (the slot of listing (e, k) is e*npos + k).
 *   SG_INCIDENCE_VE, tensor[V,E] (Link::ve, :248-276): rowptr[n+1];
 *     colidx[nE*npos] = per vertex the elements that list it, ascending,
 *     once per listing; slot_of[nE*npos] = the slot of listing (e, k).
 * Synchronises. */
enum { SG_INCIDENCE_EV = 0, SG_INCIDENCE_VE = 1 };
int sg_incidence_pattern(sg_ctx *ctx, int kind, int32_t n, int64_t nE, int32_t npos,
                         const int32_t *sel, uint32_t *rowptr, uint32_t *colidx,
                         uint32_t *slot_of);

/* Rectangular pattern ∃e.(v-e ∧ e-u) between two vertex sets of one edge
 * set (src/path_expression_analysis.cpp:80-92 with v and u in different
 * sets, e.g. matrix[V0,V1] over Set E(V1,V1,V0,V1,V1)): rows are the nr
 * vertices of the row set, reached through the elements' row-set endpoints;
 * ve_ptr / ve_idx are their incidence (sg_incidence_build over those
 * endpoints, npos_r per element); sel_c int32[nE*npos_c] the elements'
 * column-set endpoints (nc vertices).  Row v lists, sorted and unique, the
 * column-set endpoints of its elements (at most 64).  Call with colidx NULL
 * for rowptr[nr+1] and *h_nnzb, then with colidx[nnzb].  Synchronises. */
int sg_pattern_rect(sg_ctx *ctx, int32_t nr, int32_t nc, int64_t nE, int32_t npos_r,
                    int32_t npos_c, const int32_t *sel_c, const uint32_t *ve_ptr,
                    const uint32_t *ve_idx, uint32_t *rowptr, uint32_t *colidx,
                    int64_t *h_nnzb);

/* Longest row (blocks) of a pattern; synchronises.  The assembly kernels keep
 * one row image in shared memory and need this bound. */
int sg_pattern_maxrow(sg_ctx *ctx, int32_t n, const uint32_t *rowptr,
                      int32_t *h_maxrow);

/* ---------------------------------------------------------------------
 * Assembly ("map f to E reduce +").  Replaces the reference's map lowering
 * (src/inline.cpp:690-888, src/lower/lower_maps.cpp:54-128) and its GPU
 * atomics (src/backend/gpu/gpu_backend.cpp:788-846).  A group of lanes owns
 * each block row and sums its elements' contributions in ascending element
 * order (the reference's order) without atomics.  exact != 0 selects kernels
 * compiled without multiply-add contraction in the reference's operation
 * order (FP64 results equal to the reference's up to libm `log`); exact == 0
 * selects contracted kernels (and the closed-form linear-tet stiffness).
 * dtype (SG_F32 / SG_F64) is the type of every floating-point array.
 * ------------------------------------------------------------------- */

/* A bound edge set over one vertex set plus its pattern (all device). */
typedef struct sg_mesh {
  int32_t n;                  /* vertices (block rows) */
  int32_t card;               /* endpoints per element */
  int64_t nE;                 /* elements */
  const int32_t *endpoints;   /* int32[nE*card] */
  const uint32_t *ve_ptr;     /* sg_incidence_build */
  const uint32_t *ve_idx;
  const uint32_t *rowptr;     /* sg_pattern_count / sg_pattern_fill */
  const uint32_t *colidx;
  int64_t nnzb;
  int32_t maxrow;             /* sg_pattern_maxrow */
  /* Optional element-parallel assembly plans (assembly with exact == 0
   * computes every element once; exact == 1 always runs the row-owner
   * kernels, the reference's element order bit for bit; NULL / 0 everywhere:
   * row owners).  Both need slots.
   *  - slot_src_ptr / slot_src set (sg_slot_sources): element blocks are
   *    written once, then every slot sums its blocks in ascending element
   *    order and every vertex its vector contributions (deterministic).
   *  - else color_order / color_ptr set (sg_element_coloring): blocks are
   *    added into their slots colour by colour (no two elements of a colour
   *    share a vertex, so no atomics; deterministic, colour order). */
  const uint32_t *slots;       /* device [nE*card*card] (sg_slots_build) */
  const uint32_t *color_order; /* device [nE] (sg_element_coloring) */
  const int32_t *color_ptr;    /* HOST [ncolors+1]: colour k is
                                  color_order[color_ptr[k] .. color_ptr[k+1]) */
  int32_t ncolors;
  const uint32_t *slot_src_ptr; /* device [nnzb+1] (sg_slot_sources) */
  const uint32_t *slot_src;     /* device [nE*card*card] */
  int32_t asm_tile;             /* element tile of the element-blocks plan: threads
                                   per CTA, 128 / 256 / 512 (0 = 256); the host
                                   runtime's assembly tuner picks it */
} sg_mesh;

/* The inverse slot map for the element-blocks plan: for slot q, the element
 * blocks (e*card + i)*card + j with slots[...] == q, ascending, at
 * slot_src[slot_src_ptr[q] .. slot_src_ptr[q+1]).  Needs m->slots (and
 * nnzb).  Replaces the per-element `loc` searches of the reference's map
 * lowering (src/inline.cpp:524-577, src/runtime.cpp:19-23) with a gather. */
int sg_slot_sources(sg_ctx *ctx, const sg_mesh *m, uint32_t *slot_src_ptr, uint32_t *slot_src);

/* Element colouring for the plan above: no two elements of a colour share a
 * vertex (Jones-Plassmann with hashed priorities, deterministic).
 * color_order (device [nE]) receives the elements colour by colour,
 * ascending index within a colour; color_ptr (HOST, SG_MAX_COLORS + 1
 * entries) the colour offsets; *h_ncolors the colour count.  Needs the mesh's
 * endpoints and incidence; synchronises.  No counterpart in the reference,
 * whose GPU backend adds element blocks with float atomics
 * (src/backend/gpu/gpu_backend.cpp:788-846). */
#define SG_MAX_COLORS 128
int sg_element_coloring(sg_ctx *ctx, const sg_mesh *m, uint32_t *color_order,
                        int32_t *color_ptr, int32_t *h_ncolors);

enum { SG_MODEL_LINEAR = 0, SG_MODEL_NEOHOOKEAN = 1 };

/* Springs: compute_mass_damping over points + compute_elasticity over springs,
 * MDK = MD + K and f = fmg + fe (apps/springs/isprings.sim:21-68 as form 0;
 * test/input/program/isprings.sim as form 1).  x, v [n*3], mass [n],
 * fixed uint8 [n]; k, l0 [nE]; h_grav host double[3].  vals [nnzb*9], f [n*3]. */
int sg_assemble_springs(sg_ctx *ctx, const sg_mesh *mesh, int dtype, int form,
                        const void *x, const void *v, const void *mass,
                        const uint8_t *fixed, const void *k, const void *l0,
                        double h, double viscous, const double *h_grav,
                        void *vals, void *f, int exact);

/* Scalar springs of test/input/program/cg.sim: blocks +-a, then
 * A = diag*I + scale*K on the spring pattern.  a [nE], vals [nnzb]. */
int sg_assemble_scalar_springs(sg_ctx *ctx, const sg_mesh *mesh, int dtype,
                               const void *a, double diag, double scale,
                               void *vals, int exact);

/* Generic `map f to E reduce +` for a caller-evaluated element function
 * (src/lower/lower_maps.cpp:54-128; src/inline.cpp:690-888): eb holds
 * nE*card*card blocks of bs*bs values, block (i, j) of element e at
 * ((e*card + i)*card + j)*bs*bs, row-major, zero where the function writes
 * nothing; each is added into the slot of (endpoint i, endpoint j) of the
 * mesh's pattern, in element order (so FP64 sums are the reference's).
 * bs 1..3, card 2..4.  exact = 1: no contraction (parity mode). */
int sg_assemble_blocks(sg_ctx *ctx, const sg_mesh *mesh, int dtype, int bs, const void *eb,
                       void *vals, int exact);

/* `map f to E reduce +` into an incidence matrix (sg_incidence_pattern):
 * eb[(e*npos + k)*bs*bs] is the bs x bs block the element function writes at
 * (endpoint k, e) for VE or (e, endpoint k) for EV, zero where it writes
 * nothing.  Each is added, in ascending k from zero, into the first slot of
 * its (row, column) -- the slot `loc` finds -- so a repeated endpoint's
 * second slot holds zero.  vals [nE*npos*bs*bs]; bs 1..4. */
int sg_assemble_incidence(sg_ctx *ctx, int kind, int64_t nE, int32_t npos, const int32_t *sel,
                          const uint32_t *slot_of, int dtype, int32_t bs, const void *eb,
                          void *vals);

/* `map f to E reduce +` into a rectangular pattern (sg_pattern_rect):
 * eb[((e*npos_r + k)*npos_c + j)*bs*bs] is the block written at (row-set
 * endpoint k, column-set endpoint j) of element e; each row owner adds them
 * in ascending (e, k, j) from zero.  vals [nnzb*bs*bs]; bs 1..4. */
int sg_assemble_rect(sg_ctx *ctx, int32_t nr, int32_t npos_r, int32_t npos_c,
                     const int32_t *sel_c, const uint32_t *ve_ptr, const uint32_t *ve_idx,
                     const uint32_t *rowptr, const uint32_t *colidx, int dtype, int32_t bs,
                     const void *eb, void *vals);

/* Element kernels compiled at run time (NVRTC, loaded on first use): the
 * element function of a `map f to E reduce +` given as CUDA C++ source,
 *   __device__ int element_block(long long e, int i, int j, const int *ep,
 *                                const real *const *f, sg_block *blk);
 * (real = float or double per dtype; BS, CARD, SG_TERMS = 2 defined and
 * sg_block = real[BS][BS]; ep the element's endpoints; f the fields passed
 * to sg_jit_assemble, cast by the source where a field is not real).  It
 * writes the terms element e adds to block (i, j) into blk[0..] and returns
 * their count (0 .. SG_TERMS); each term is its own `+=` on the slot, as
 * each write of the reference's element function is after lowering.  The
 * source is compiled with a row-owner assembly kernel for sm_103a (exact !=
 * 0: no multiply-add contraction) that adds, per slot and from zero, in
 * ascending element order, then ascending j, then term, as sg_assemble_blocks
 * does for precomputed blocks.  This is the code-generation end of the
 * reference's map lowering (src/inline.cpp:690-888,
 * src/lower/lower_maps.cpp:54-128) with the element function written in
 * CUDA rather than produced from .sim by its frontend.  card 1..32, bs 1..16
 * (a nested block type is one flat block: 3x3 blocks of 3x3 are bs 9); a
 * row must fit the kernel's 48 KB of shared memory, else sg_jit_assemble
 * returns SG_ERR_UNSUPPORTED.  A source that does not compile returns SG_ERR_ARG with the compiler log in
 * sg_last_error(); without NVRTC, SG_ERR_UNSUPPORTED. */
typedef struct sg_jit_assembly sg_jit_assembly;
/* Compiles the source as sg_jit_assembly_create does, without a context or
 * a GPU; the compiler log (warnings or errors) goes to log[log_cap]. */
int sg_jit_check_source(const char *element_src, int32_t card, int32_t bs, int dtype,
                        int32_t exact, char *log, int64_t log_cap);
int sg_jit_assembly_create(sg_ctx *ctx, const char *element_src, int32_t card, int32_t bs,
                           int dtype, int32_t exact, sg_jit_assembly **out);
/* h_fields: host array of nfields (<= 8) device pointers; vals [nnzb*bs*bs]. */
int sg_jit_assemble(sg_jit_assembly *jit, const sg_mesh *mesh, const void *const *h_fields,
                    int32_t nfields, void *vals);
int sg_jit_assembly_destroy(sg_jit_assembly *jit);
/* The same for a map whose result is a system vector: the source defines
 *   __device__ int element_vector(long long e, int i, const int *ep,
 *                                 const real *const *f, sg_vec *vec);
 * (sg_vec = real[BS], at most SG_VTERMS = 8 terms) writing the terms
 * element e adds to its endpoint i.  sg_jit_assemble_vector writes
 * vals [n*bs]: each vertex adds, from zero, its incidences' terms in
 * ascending (element, local index), each element's terms in its order (the
 * lowered map's `+=` per write).  The handle is destroyed with
 * sg_jit_assembly_destroy. */
int sg_jit_check_vector_source(const char *element_src, int32_t card, int32_t bs, int dtype,
                               int32_t exact, char *log, int64_t log_cap);
int sg_jit_vector_create(sg_ctx *ctx, const char *element_src, int32_t card, int32_t bs,
                         int dtype, int32_t exact, sg_jit_assembly **out);
int sg_jit_assemble_vector(sg_jit_assembly *jit, const sg_mesh *mesh,
                           const void *const *h_fields, int32_t nfields, void *vals);

/* The cloth example's forces (apps/cloth/cloth.sim) as system vectors
 * f [n*3] (`map ... to faces / hinges reduce +`), each vertex summing from
 * zero its incidences' terms in ascending (element, local index), each
 * element's terms in the program's order; no multiply-add contraction.
 * sg_assemble_cloth_stretch: stretchingForce (:142-164) over faces (card 3),
 * K [nF*9] the per-face stretching matrix (row-major), rest [nF*3] the rest
 * squared lengths of edges 0-1, 1-2, 2-0 (precomputeFaceQuantities).
 * sg_assemble_cloth_bend: bendingForce (:166-173) over hinges (card 4: the
 * shared edge's endpoints, then the opposite vertices of its two
 * triangles), angle / len / perp [nH] the rest dihedral angle, the edge's
 * rest length and 2 (A1 + A2) / (3 len) (precomputeHingeQuantities).
 * x [n*3]; all arrays in dtype.  Asynchronous. */
int sg_assemble_cloth_stretch(sg_ctx *ctx, const sg_mesh *faces, int dtype, const void *x,
                              const void *K, const void *rest, void *f);
int sg_assemble_cloth_bend(sg_ctx *ctx, const sg_mesh *hinges, int dtype, const void *x,
                           const void *angle, const void *len, const void *perp, void *f);

/* precomputeTetMat (femTet.sim; apps/fem/fem_linear.sim:176-193):
 * B = inv(Ds) [nE*9], W = -det(Ds)/6 [nE], vertex mass m [n] = sum of
 * 0.25*rho*W in element order. */
int sg_tet_precompute(sg_ctx *ctx, const sg_mesh *mesh, int dtype,
                      const void *x, double rho, void *B, void *W, void *mass);

/* compute_stiffness of femTet.sim (SG_MODEL_NEOHOOKEAN: dPdF tangent) or of
 * apps/fem/fem_linear.sim:105-174 (SG_MODEL_LINEAR: W*B'*E*B), scaled by h*h,
 * plus the lumped element mass on the diagonal; c int32 [n] (c > 0 =
 * constrained); mu, lam [nE].  The neo-Hookean path uses nE*16*9 values of
 * context scratch. */
int sg_assemble_tet_stiffness(sg_ctx *ctx, const sg_mesh *mesh, int dtype,
                              int model, const void *x, const int32_t *c,
                              const void *B, const void *W, const void *mu,
                              const void *lam, double h, double rho,
                              void *vals, int exact);

/* compute_force of femTet.sim / fem_linear.sim:55-93; f [n*3]. */
int sg_assemble_tet_force(sg_ctx *ctx, const sg_mesh *mesh, int dtype,
                          int model, const void *x, const void *v,
                          const int32_t *c, const void *B, const void *W,
                          const void *mu, const void *lam, double h,
                          double rho, const double *h_grav, void *f, int exact);

/* P1 heat, backward Euler: A = M + dt*K(kappa), b = M*T0 (scalar blocks);
 * kappa [nE], T0 [n], vals [nnzb], b [n]. */
int sg_assemble_heat(sg_ctx *ctx, const sg_mesh *mesh, int dtype,
                     const void *B, const void *W, const void *kappa,
                     double dt, const void *T0, void *vals, void *b, int exact);

/* ---------------------------------------------------------------------
 * Blocked SpMV  y = A x.  Replaces the lowered SpMV loop nest
 * (src/lower/index_expressions/lower_indexexprs.cpp:630-660).
 * bs = 1, 2, 3 have dedicated kernels; other bs use a generic kernel.
 * val_dtype is the matrix value type; vec_dtype the type of x and y;
 * accumulation is in the wider of the two.  g = 1,2,4,8,16,32 selects the
 * streaming kernel with g lanes per block row; g = -1..-15 selects variant
 * -g-1 of the TMA-staged kernel (bs = 3, 16-byte aligned vals/colidx;
 * variants differ in lanes per row, rows per tile, pipeline stages and
 * whether a CTA or each warp runs the copy pipeline; a variant whose
 * buffers cannot hold the pattern's largest tile runs the streaming kernel);
 * g = 0 picks (the default TMA variant for FP32 values, the streaming kernel
 * for FP64).
 * ------------------------------------------------------------------- */
int sg_bspmv(sg_ctx *ctx, int32_t n, int32_t bs, const uint32_t *rowptr,
             const uint32_t *colidx, int val_dtype, const void *vals,
             int vec_dtype, const void *x, void *y, int32_t g);

/* y = y + alpha * x (two separately rounded operations, as the lowered
 * `points.x = points.x + h * points.v` of apps/springs/isprings.sim:94 and
 * `verts.x = h * x + verts.x` of femTet.sim); vec_dtype for x and y. */
int sg_axpy(sg_ctx *ctx, int64_t len, int vec_dtype, double alpha, const void *x, void *y);

/* Symmetric storage of a 3x3-blocked FP32 matrix (the layout the solver's
 * SG_STORAGE_SYMMETRIC option iterates on).  create: from a full pattern that
 * is symmetric, sorted and has every diagonal block, builds the upper-half
 * CSR and, per row, the index {column, upper slot} of its blocks below the
 * diagonal (synchronises; SG_ERR_DEVICE for a missing diagonal block or an
 * asymmetric pattern).  fill: copies the upper blocks out of full values
 * [nnzb*9] (the lower ones are not read).  spmv: y = A x with A the
 * symmetric matrix whose upper half was filled; FP32 x, y [n*3].  The
 * reference has no symmetric storage: it always reads full blocked CSR
 * (src/lower/index_expressions/lower_indexexprs.cpp:630-665). */
typedef struct sg_symbsr sg_symbsr;
int sg_symbsr_create(sg_ctx *ctx, int32_t n, const uint32_t *rowptr, const uint32_t *colidx,
                     int64_t nnzb, int32_t stages /* bulk-copy stages 2..4, 0 = default */,
                     sg_symbsr **out);
int sg_symbsr_fill(sg_symbsr *s, const float *vals);
int sg_symbsr_spmv(sg_symbsr *s, const float *x, float *y);
int sg_symbsr_destroy(sg_symbsr *s);

/* System-matrix expression out = D + scale*K on K's pattern (replaces the
 * lowered `MDK = MD + K` of apps/springs/isprings.sim:74, with the storage
 * rules of src/storage.cpp:358-360 and 416-470).  D is Diagonal storage:
 * diag [n*bs*bs] (block of vertex v at v*bs*bs, row-major), or, with diag
 * NULL, ident*I (ident = 0: no diagonal term, out = 0 + scale*K).  A diagonal
 * slot holds D + (scale*K), every other slot 0 + (scale*K), each operation
 * rounded separately in dtype.  out may alias vals.  Asynchronous; a row
 * without its diagonal block, when D is given, fails the next sg_ctx_sync. */
int sg_bsr_add_diag(sg_ctx *ctx, int32_t n, int32_t bs, const uint32_t *rowptr,
                    const uint32_t *colidx, int64_t nnzb, int dtype, const void *diag,
                    double ident, double scale, const void *vals, void *out);

/* Dot product of two blocked vectors with an FP64 deterministic two-level
 * reduction; synchronises. */
int sg_dot(sg_ctx *ctx, int64_t len, int vec_dtype, const void *a,
           const void *b, double *h_out);

/* The device's FP64 FMA rate in TFLOP/s (2 flops per FMA), from a kernel of
 * independent FMA chains on every SM, timed on the context's stream: the
 * FP64 roofline of an FP64 SpMV.  Synchronises. */
int sg_fp64_fma_rate(sg_ctx *ctx, double *tflops);

/* ---------------------------------------------------------------------
 * Conjugate-gradient solves.  The reference has no CG routine: CG is user
 * code in each .sim program (apps/springs/isprings.sim:77-93,
 * apps/fem/fem_linear.sim:211-230, test/input/program/cg.sim:25-53, Jacobi
 * PCG apps/thermal/thermal.sim:102-130).  These entry points replace those
 * loops with fused kernels (SpMV + dot, update + preconditioner + dots,
 * direction) captured in a CUDA graph, with FP64 deterministic reductions.
 *
 * precision SG_SOLVE_F64: matrix, vectors and reductions in FP64.
 * precision SG_SOLVE_MIXED: SpMV and vector bulk in FP32 (matrix stored in
 *   FP32), dots in FP64, and FP64 reliable updates: whenever the iterated
 *   residual has dropped by reliable_delta (or says "converged"), x_hi +=
 *   x_lo and r = b - A x_hi are recomputed in FP64 and the iteration
 *   continues from the true residual (outer iterative refinement without a
 *   Krylov restart).
 * stop: SG_STOP_NORMR2 (r'r <= tol, isprings.sim / femTet.sim),
 *   SG_STOP_NORMR (||r|| <= tol, cg.sim), SG_STOP_RELATIVE (||r|| <=
 *   tol*||b||, thermal.sim).
 * verify = 0 ends when the iterated residual passes, as the reference loops
 *   do; verify = 1 confirms with the true FP64 residual and continues if it
 *   does not pass.
 * check_every > 0 replaces r by b - A x every check_every iterations
 *   (thermal.sim's mod(iter,50) refresh).
 * ------------------------------------------------------------------- */
enum { SG_SOLVE_F64 = 0, SG_SOLVE_MIXED = 1 };
enum {
  SG_PRECOND_NONE = 0,
  SG_PRECOND_JACOBI = 1,        /* point Jacobi (thermal.sim assemble_jacobi) */
  SG_PRECOND_BLOCK_JACOBI = 2,  /* inverse of each 3x3 diagonal block */
  SG_PRECOND_LEARNED = 3        /* message-passing network (sg_mpnn_*) in flexible
                                   PCG; needs SG_SOLVE_MIXED and bs = 3.  Falls back
                                   to block Jacobi when r.z <= 0 or the residual
                                   grows 100x (result.fallbacks counts it). */
};
enum { SG_STOP_NORMR2 = 0, SG_STOP_NORMR = 1, SG_STOP_RELATIVE = 2 };
enum {
  SG_STATUS_CONVERGED = 1,
  SG_STATUS_MAXITER = 2,
  SG_STATUS_BREAKDOWN = 3,      /* p'Ap <= 0 */
  SG_STATUS_NAN = 4
};

/* A blocked-CSR system matrix (device arrays). */
typedef struct sg_matrix {
  int32_t n;                 /* block rows */
  int32_t bs;                /* block size */
  int64_t nnzb;
  const uint32_t *rowptr;
  const uint32_t *colidx;
  int dtype;                 /* type of vals */
  const void *vals;
} sg_matrix;

/* SpMV autotuner: times y = A x (x of xdt) on the matrix itself with every
 * candidate schedule sg_bspmv accepts -- the default (g = 0), every TMA
 * variant (per-warp or CTA tiles, lanes per block row, pipeline stages; g < 0)
 * and every streaming lane count (g = 1..32) -- reps calls each, and returns
 * the fastest g and its time (*default_ms: the default's).  The choice is
 * cached per (device, n, nnzb, bs, dtypes, pattern arrays); a cached choice
 * is returned at once (*ncand = 0) unless force.  cand_g / cand_ms (cand_cap
 * entries, optional) receive every candidate's time.  Synchronises.  Replaces
 * the reference GPU backend's fixed 16-thread blocks
 * (src/backend/gpu/gpu_backend.h:49-51). */
int sg_tune_spmv(sg_ctx *ctx, const sg_matrix *A, int xdt, int reps, int force,
                 int32_t *best_g, float *best_ms, float *default_ms, int32_t *ncand,
                 int32_t *cand_g, float *cand_ms, int32_t cand_cap);
/* sg_solve_opts.lanes = SG_LANES_AUTOTUNE: the solver takes its SpMV
 * schedule from sg_tune_spmv at set-up. */
#define SG_LANES_AUTOTUNE 1000

/* Storage the iteration's SpMV reads.  SG_STORAGE_SYMMETRIC keeps the blocks
 * on and above the diagonal plus an index of the blocks below it (see
 * sg_symbsr_create); the matrix must be symmetric bit for bit, as the tet
 * stiffness maps assemble it.  The true residual still uses the full matrix. */
enum { SG_STORAGE_FULL = 0, SG_STORAGE_SYMMETRIC = 1 };

typedef struct sg_solve_opts {
  int precision;             /* SG_SOLVE_F64 / SG_SOLVE_MIXED */
  int precond;               /* SG_PRECOND_* */
  int stop;                  /* SG_STOP_* */
  double tol;
  int32_t maxiters;
  int32_t verify;
  int32_t check_every;
  double reliable_delta;     /* mixed only; 0 -> 0.1 */
  int32_t lanes;             /* SpMV lanes per block row; 0 = default */
  int32_t batch;             /* iterations per graph launch (even); 0 = 32 */
  const float *learned_params; /* SG_PRECOND_LEARNED: device FP32[sg_mpnn_nparams()] */
  int32_t learned_form;        /* SG_MPNN_RELU / SG_MPNN_LINEAR / SG_MPNN_SYM */
  int32_t storage;             /* SG_STORAGE_FULL / SG_STORAGE_SYMMETRIC (mixed, bs 3):
                                  the iteration's SpMV reads the upper half only */
  int32_t pdl;                 /* 1: programmatic dependent launch between the
                                  iteration's kernels in the captured graph (the
                                  next kernel launches while its predecessor
                                  drains); 0 (default): plain graph edges, which
                                  measured 4 % faster at 128^3 */
  int32_t learned_exec;        /* SG_MPNN_SYM: SG_MPNN_EXEC_FOLDED (default),
                                  SG_MPNN_EXEC_FOLDED_F32 or SG_MPNN_EXEC_LAYERED
                                  (see sg_mpnn_graph_set_exec); the other forms
                                  always run layered */
} sg_solve_opts;

typedef struct sg_solve_result {
  int32_t status;            /* SG_STATUS_* */
  int32_t iters;
  int32_t checks;            /* true-residual checks / reliable updates */
  int32_t fallbacks;         /* learned preconditioner -> Jacobi switches */
  double normr2;             /* last iterated r'r */
  double true_normr2;        /* ||b - A x||^2 at exit (FP64) */
  double bnorm2;             /* b'b */
  int64_t kernels;           /* kernels this solve launched (graph nodes included) */
} sg_solve_result;

typedef struct sg_solver sg_solver;

/* Set-up: workspace, the FP32 matrix copy (mixed with FP64 input), the
 * preconditioner and the captured iteration graph. */
int sg_solver_create(sg_ctx *ctx, const sg_matrix *A, const sg_solve_opts *opts,
                     sg_solver **out);
/* Solve A x = b; b, x FP64 device arrays of n*bs; x holds the initial guess
 * and receives the solution.  Synchronises. */
int sg_solver_solve(sg_solver *s, const double *b, double *x, sg_solve_result *res);
/* The same with a right-hand side of either precision (b_dtype SG_F32 or
 * SG_F64; an FP32 b, e.g. the force map of an FP32 assembly, is widened by
 * the solver's own kernel into an FP64 copy it keeps) and, with x_zero = 1,
 * the zero initial guess (x is only written).  Lets an assembly + solve step
 * run without a separate conversion or fill. */
int sg_solver_solve_ex(sg_solver *s, const void *b, int b_dtype, double *x, int x_zero,
                       sg_solve_result *res);
/* Re-read the matrix values after they changed in place (re-assembly):
 * refreshes the FP32 bulk copy and the (block-)Jacobi diagonal; the captured
 * iteration graph is kept. */
int sg_solver_refresh(sg_solver *s);
int sg_solver_destroy(sg_solver *s);
/* One-shot create + solve + destroy. */
int sg_solve(sg_ctx *ctx, const sg_matrix *A, const sg_solve_opts *opts,
             const double *b, double *x, sg_solve_result *res);

/* True residual r = b - A x (FP64 x, b, r [n*bs]) and h_rr = ||r||^2;
 * synchronises.  mode SG_RESIDUAL_FP64: FP64 accumulation (any bs and
 * dtype).  SG_RESIDUAL_COMPENSATED (FP32 3x3 matrices): x split into float
 * pairs and compensated FP32 products and sums, about 2^-46 of sum |A||x|
 * accurate, without FP64 multiply-adds (the solver's checks between
 * residual replacements).  The reference computes residuals in its .sim
 * programs (apps/thermal/thermal.sim:88-93) with the lowered SpMV. */
enum { SG_RESIDUAL_FP64 = 0, SG_RESIDUAL_COMPENSATED = 1 };
int sg_residual(sg_ctx *ctx, const sg_matrix *A, const double *x, const double *b, double *r,
                double *h_rr, int mode);

/* ---------------------------------------------------------------------
 * Batched PCG: nsys independent 3x3-blocked systems concatenated into one
 * block-diagonal FP32 matrix (system s = block rows [sys_ptr[s],
 * sys_ptr[s+1]), columns inside that range only), solved in ONE persistent
 * launch: each CTA takes whole systems from a queue in the given order
 * (`order`, largest first for load balance) and runs mixed-precision
 * block-Jacobi PCG on them with CTA-local barriers only.  Each system stops
 * at ||b_s - A_s x_s|| <= tol ||b_s|| (confirmed in FP64) or maxiters.
 * b, x FP32 [n*3] device (x: guess in, solution out); iters, status
 * (SG_STATUS_*), relres per system (device).  config selects threads per
 * CTA and lanes per row (0 .. sg_batched_configs()-1; the autotuner in the
 * host runtime picks one).  Asynchronous; capturable after a first call has
 * sized the context scratch.  Replaces running one Simit program per mesh
 * (no batched counterpart in the reference).
 * ------------------------------------------------------------------- */
int sg_batched_pcg(sg_ctx *ctx, int32_t nsys, const int32_t *sys_ptr, const int32_t *order,
                   const sg_matrix *A, const float *b, float *x, double tol,
                   int32_t maxiters, int32_t config, int32_t *iters, int32_t *status,
                   double *relres);
int sg_batched_configs(void);

/* ---------------------------------------------------------------------
 * Locality reordering (host; simit::reorder, src/reorder.cpp:252-273).
 * sg_hilbert_order: vertex_ordering[old] = new index of each vertex, by the
 * Hilbert index of its cell, cell = floor((x - min) 2^bits / extent) in
 * 0 .. 2^bits per axis (the curve spans 2^(bits+1) cells, so the upper
 * faces come last; bits 1..20; ties by old index).  sg_element_order: element_order[new] = old index,
 * elements sorted by their sorted endpoint tuples (apply after relabelling
 * the endpoints).  sg_hilbert_index exposes the curve for tests.
 * ------------------------------------------------------------------- */
int sg_hilbert_order(int32_t n, const double *coords, int32_t bits, int32_t *vertex_ordering);
/* The same with the Morton (Z-order) curve (no counterpart in the reference). */
int sg_morton_order(int32_t n, const double *coords, int32_t bits, int32_t *vertex_ordering);
int sg_element_order(int32_t nE, int32_t card, const int32_t *endpoints, int32_t *element_order);
int sg_hilbert_index(uint32_t x, uint32_t y, uint32_t z, int32_t bits, uint64_t *out);

/* ---------------------------------------------------------------------
 * Learned preconditioner: a 3-layer message-passing network (hidden 64,
 * messages of 8, no biases) over the matrix graph, z = D^-1 r + Wout h3,
 * where D is the 3x3 block diagonal; the 64x64 layers run on the tensor
 * cores with bf16 weights and FP32 accumulation.  It has no counterpart in
 * the reference (it preconditions the flexible PCG).  Three forms
 * (SG_MPNN_*): relu activations; identity activations (z linear in r); and
 * the symmetric factorized form M = L^-T (I+N)^T (I+N) L^-1 of the linear
 * network N with D = L L^T per vertex, symmetric positive definite by
 * construction and equal to block Jacobi when Wout = 0 ((I+N)^T runs as the
 * same layers with transposed weights).  Parameters are one flat
 * FP32 device array of sg_mpnn_nparams() values.  Training: forward with
 * train = 1 keeps activations, sg_mpnn_loss gives the A-norm error
 * (z-e)'A(z-e)/e'Ae of a residual/correction pair (r, e = A^-1 r) and dL/dz,
 * sg_mpnn_backward the parameter gradient, sg_mpnn_adam the update.
 * ------------------------------------------------------------------- */
typedef struct sg_mpnn_graph sg_mpnn_graph;
int sg_mpnn_nparams(void);
/* Edge weights and block-Jacobi of a 3x3-blocked matrix (FP32 or FP64). */
int sg_mpnn_graph_create(sg_ctx *ctx, const sg_matrix *A, sg_mpnn_graph **out);
int sg_mpnn_graph_refresh(sg_mpnn_graph *g);
enum { SG_MPNN_RELU = 0, SG_MPNN_LINEAR = 1, SG_MPNN_SYM = 2 };
/* Select the form (default SG_MPNN_RELU). */
int sg_mpnn_graph_set_form(sg_mpnn_graph *g, int form);
/* How sg_mpnn_forward (train = 0) evaluates the symmetric form.  With
 * identity activations every hidden layer is a fixed linear map of the
 * inputs and messages before it and commutes with the edge-weight
 * aggregation Aw, so M = L^-T [sum_{d=0..6} Aw^d (x) G_d] L^-1 with 3x3
 * coefficients G_d (computed in FP64 from the same bf16-rounded 64x64
 * weights): one application is six Horner gather passes of 3-wide vectors
 * over a sliced-ELLPACK copy of the pattern.  SG_MPNN_EXEC_FOLDED stores
 * the edge weights as FP16 and x and the Horner sums in per-vertex block
 * floating point (FP16 mantissas, a shared power-of-two exponent);
 * SG_MPNN_EXEC_FOLDED_F32 keeps both in FP32; SG_MPNN_EXEC_LAYERED (the
 * default here) runs the tensor-core layers.  Training always runs
 * layered.  The folded evaluations need r and z 16-byte aligned. */
enum { SG_MPNN_EXEC_FOLDED = 0, SG_MPNN_EXEC_LAYERED = 1, SG_MPNN_EXEC_FOLDED_F32 = 2 };
int sg_mpnn_graph_set_exec(sg_mpnn_graph *g, int exec);
/* One Horner step (d = 5 .. 0) of the folded evaluation on the graph's own
 * buffers, as the last folded sg_mpnn_forward left them: step 5 gathers x,
 * step d < 5 the sums step d + 1 wrote.  For timing a pass on its own; the
 * graph's folded buffers must exist (a folded forward ran). */
int sg_mpnn_fold_step(sg_mpnn_graph *g, int32_t d);
int sg_mpnn_graph_destroy(sg_mpnn_graph *g);
/* z = M(r); r, z FP32 [n*3]. */
int sg_mpnn_forward(sg_mpnn_graph *g, const float *params, const float *r, float *z,
                    int train);
/* grad (FP32[nparams], overwritten) of <dz, M(r)> for the r of the last
 * train-mode forward. */
int sg_mpnn_backward(sg_mpnn_graph *g, const float *params, const float *dz, float *grad);
/* A-norm loss of z against e (FP32 matrix graphs); dz = 2 A (z-e) / e'Ae. */
int sg_mpnn_loss(sg_mpnn_graph *g, const float *z, const float *e, double eAe, float *dz,
                 double *h_loss);
int sg_mpnn_adam(sg_ctx *ctx, float *params, const float *grad, float *m, float *v, int step,
                 float lr, float beta1, float beta2, float eps);

/* ---------------------------------------------------------------------
 * Dot product that allocates nothing.  This entry point has no counterpart
 * in the reference; it exists for callers that may not allocate device
 * memory while they run -- a host application that owns and budgets all GPU
 * memory through its own pool, or a time-critical loop that must not call
 * cudaMalloc/cudaFree because those can synchronise the device.  Such a
 * caller cannot create an sg_ctx (its set-up allocates) or use sg_dot (its
 * partial sums live in the context's growable scratch arena).
 *
 * FP64 accumulation in a fixed order (deterministic for a given len; sums
 * are split by 4096-element chunks, so the last bits may differ from
 * sg_dot's), computed on `stream` (a cudaStream_t of the current device, NULL
 * = legacy default stream) into the caller's DEVICE double *d_out,
 * asynchronously.  The partial sums live in a
 * fixed static device array (SG_DOT_NOALLOC_MAX_PARTS doubles, 512 KB, held
 * by every GPU that loads the library until exit), so len is limited to
 * SG_DOT_NOALLOC_MAX_LEN elements; longer vectors are rejected with
 * SG_ERR_ARG.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) while that device is current and loads the
 * kernels, which may allocate once; make it before any stream capture and
 * before the stretch that must not allocate.  Calls share the array: calls
 * whose kernels may overlap on the GPU (unordered streams) race, so order
 * them on one stream.
 * ------------------------------------------------------------------- */
#define SG_DOT_NOALLOC_CHUNK 4096
#define SG_DOT_NOALLOC_MAX_PARTS 65536
#define SG_DOT_NOALLOC_MAX_LEN ((int64_t)SG_DOT_NOALLOC_CHUNK * SG_DOT_NOALLOC_MAX_PARTS)
int sg_dot_noalloc(void *stream, int64_t len, int vec_dtype, const void *a,
                   const void *b, double *d_out);

#ifdef __cplusplus
}
#endif
#endif /* SIMIT_GB300_H */
