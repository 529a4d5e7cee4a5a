// Symmetric storage of a 3x3-blocked FP32 matrix with a symmetric pattern:
// only the blocks on and above the diagonal are kept (upper CSR, `uvals`),
// and each row lists its blocks below the diagonal as (column c, upper slot
// of block (c, r)), whose transpose they are.  The SpMV streams the upper
// half (36 value bytes + 4 index bytes per block) and 8 index bytes per lower
// block from HBM; the lower blocks' values are the upper blocks of nearby
// rows, read again from L2.  At 128^3 that is 0.77 GB per SpMV instead of
// 1.16 GB for full storage.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace sg {

struct Ctx;
struct SolveCtl;

struct SymBsr {
  Ctx *c = nullptr;
  int32_t n = 0;
  int64_t nnzb = 0, nu = 0, nl = 0;          // full, upper and lower block counts
  const uint32_t *rowptr = nullptr, *colidx = nullptr;  // the full pattern
  uint32_t *dslot = nullptr;                 // full slot of each row's diagonal block
  uint32_t *urowptr = nullptr, *ucol = nullptr, *lrowptr = nullptr;
  uint2 *lidx = nullptr;                     // lower block: {column, upper slot}
  float *uvals = nullptr;                    // nu blocks of 9 values, row-major
  int capu = 0, capl = 0;                    // blocks of the largest warp tile
  int nst = 3;                               // bulk-copy pipeline stages per warp
  int grid[2] = {0, 0};                      // [dot]: persistent grid
  size_t smem[2] = {0, 0};
  std::vector<void *> allocs;
};

// Builds the upper pattern and lower index from a full symmetric pattern
// (rows sorted, every row with its diagonal block); stages 0 = default.
// Synchronises.
int sym_create(Ctx *c, int32_t n, const uint32_t *rowptr, const uint32_t *colidx, int64_t nnzb,
               int stages, SymBsr *S);
// Copies the upper blocks out of full FP32 values [nnzb*9].
int sym_fill(SymBsr *S, cudaStream_t st, const float *vals);
// y = A x; with dot, also the CG K1 epilogue (p.q into ctl->pq_tot via part).
int sym_launch(SymBsr *S, cudaStream_t st, const SolveCtl *ctl, bool dot, const float *x,
               float *y, double *part);
void sym_free(SymBsr *S);

}  // namespace sg
