// Element assembly ("map f to E reduce +") into blocked CSR, row-owner form.
//
// The reference inlines the element function into a loop over elements in
// ascending order and `+=`s every block into the CSR slot found by `loc`
// (src/inline.cpp:690-888, src/lower/lower_maps.cpp:54-128; on its GPU
// backend the `+=` becomes atom.add.f32, src/backend/gpu/gpu_backend.cpp:
// 788-846).  Here a group of G lanes OWNS one block row v instead:
//
//   for each incidence (e, i) of v, in ascending e (the sorted incidence
//   list): the lanes compute row i of element e's blocks (lane = (j, l):
//   block column j, block row l) and add them into a shared-memory image of
//   row v at the position of column ep[e,j] (binary search of the row's
//   sorted columns); then the row is combined with the vertex-set map (the
//   reference's MD + K / I + c*K) and written once, coalesced.
//
// Consequences: no atomics, no colouring passes, every value written once,
// and each slot accumulates its contributions in ascending element order
// starting from zero -- the reference's summation order.  Kernels compiled
// with --fmad=false (the *_exact.cu instantiation) and written in the
// reference's operation order therefore reproduce its FP64 values bit for bit
// (up to `log`, which may differ by an ulp from the host libm).
//
// Per-element work is recomputed by each of its card row owners; for the
// neo-Hookean tangent, whose element blocks are expensive, a separate
// element-parallel kernel writes the blocks once to a scratch array and the
// row owners gather from it (EbGather).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace sg {

template <typename T> struct AsmArgs {
  int32_t n = 0;
  int32_t card = 0;
  int64_t nE = 0;
  const int32_t *ep = nullptr;
  const uint32_t *ve_ptr = nullptr, *ve_idx = nullptr;
  const uint32_t *rowptr = nullptr, *colidx = nullptr;
  // vertex fields
  const T *x = nullptr, *v = nullptr, *m = nullptr;
  const uint8_t *fixed = nullptr;
  const int32_t *c = nullptr;
  // element fields
  const T *k = nullptr, *l0 = nullptr, *a = nullptr;
  const T *B = nullptr, *W = nullptr, *mu = nullptr, *lam = nullptr, *kappa = nullptr;
  const T *T0 = nullptr;
  const T *eb = nullptr;  // element blocks (EbGather)
  // scalars
  T h = 0, viscous = 0, rho = 0, diag = 0, scale = 0, dt = 0;
  T grav[3] = {0, 0, 0};
  int form = 0;
  // outputs
  T *vals = nullptr, *f = nullptr;
  int *err = nullptr;
  int maxrow = 0;
  int64_t nnzb = 0;
};

// ---------------------------------------------------------------------------
// small dense helpers in the reference's operation order
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T d_det3(const T *a) {
  return a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
         a[2] * (a[3] * a[7] - a[4] * a[6]);
}
// src/runtime.cpp:147-173
template <typename T> __device__ __forceinline__ void d_inv3(const T *a, T *inv) {
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
template <typename T> __device__ __forceinline__ void d_mm3(const T *A, const T *B, T *C) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T t = 0;
#pragma unroll
      for (int k = 0; k < 3; ++k) t += A[i * 3 + k] * B[k * 3 + j];
      C[i * 3 + j] = t;
    }
}
template <typename T> __device__ __forceinline__ void d_tr3(const T *A, T *At) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) At[i * 3 + j] = A[j * 3 + i];
}
__device__ __forceinline__ float d_log(float x) { return logf(x); }
__device__ __forceinline__ double d_log(double x) { return log(x); }
__device__ __forceinline__ float d_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double d_sqrt(double x) { return sqrt(x); }
// Separately rounded products and sums (never contracted into a multiply-add).
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// ---------------------------------------------------------------------------
// Row-owner kernel
// ---------------------------------------------------------------------------
// Elem provides (all __device__ static):
//   int block(const AsmArgs<T>&, int64_t e, int i, int j, int l, T out[2][BS])
//       row l of block (i, j) of element e as up to two terms that are added
//       one after the other (the element function's separate `+=` writes to
//       that block, in statement order); returns the number of terms
//   int vec(const AsmArgs<T>&, int64_t e, int i, int l, T out[4])
//       the same for component l of the vector contribution to local vertex i
//   T    fin_block(const AsmArgs<T>&, int32_t v, bool diag, int l, int m, T acc)
//   T    fin_vec(const AsmArgs<T>&, int32_t v, int l, T acc)
//   constexpr HAS_MAT, HAS_VEC, LANES (= card * BS lanes used per incidence)
template <class Elem, int G, int BS, typename T>
__global__ void __launch_bounds__(128) k_rows(AsmArgs<T> a) {
  extern __shared__ unsigned char smem_raw[];
  const int groups = blockDim.x / G;
  const int grp = threadIdx.x / G;
  const int gl = threadIdx.x % G;
  const unsigned gmask = (G == 32) ? 0xffffffffu
                                   : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  const int maxrow = a.maxrow;
  T *acc = reinterpret_cast<T *>(smem_raw) + (size_t)grp * maxrow * BS * BS;
  uint32_t *cols = reinterpret_cast<uint32_t *>(reinterpret_cast<T *>(smem_raw) +
                                                (size_t)groups * maxrow * BS * BS) +
                   (size_t)grp * maxrow;
  const int64_t stride = (int64_t)gridDim.x * groups;
  for (int64_t v = (int64_t)blockIdx.x * groups + grp; v < a.n; v += stride) {
    uint32_t r0 = 0, rlen = 0;
    if (Elem::HAS_MAT) {
      r0 = a.rowptr[v];
      rlen = a.rowptr[v + 1] - r0;
      if ((int)rlen > maxrow) {
        if (gl == 0) atomicCAS(a.err, 0, 4 /* DEV_ROW_OVERFLOW */);
        continue;
      }
      for (uint32_t q = gl; q < rlen; q += G) cols[q] = a.colidx[r0 + q];
      for (uint32_t q = gl; q < rlen * BS * BS; q += G) acc[q] = T(0);
    }
    T vacc = T(0);
    __syncwarp(gmask);
    const uint32_t i0 = a.ve_ptr[v], i1 = a.ve_ptr[v + 1];
    for (uint32_t it = i0; it < i1; ++it) {
      const uint32_t t = a.ve_idx[it];
      const int64_t e = t / (uint32_t)a.card;
      const int i = (int)(t - (uint32_t)e * a.card);
      if (Elem::HAS_MAT && gl < Elem::LANES) {
        const int j = gl / BS, l = gl % BS;
        const uint32_t col = (uint32_t)a.ep[e * a.card + j];
        // An element that lists the same vertex twice sends blocks (i, j)
        // and (i, j2) to one slot: the lane of the first such j adds them
        // all, in ascending j (the reference's order), and the others skip.
        bool first = true, dup = false;
        constexpr int CARD = Elem::LANES / BS;  // every matrix element uses card * BS lanes
#pragma unroll
        for (int j2 = 0; j2 < CARD; ++j2) {
          const bool same = j2 != j && (uint32_t)a.ep[e * a.card + j2] == col;
          dup = dup || same;
          first = first && !(same && j2 < j);
        }
        if (!dup) {  // the usual case: one block per slot
          T out[2][BS];
          const int nt = Elem::block(a, e, i, j, l, out);
          if (nt > 0) {
            uint32_t lo = 0, hi = rlen;
            while (lo < hi) {
              uint32_t mid = (lo + hi) >> 1;
              if (cols[mid] < col) lo = mid + 1; else hi = mid;
            }
            T *dst = acc + (size_t)lo * BS * BS + l * BS;
#pragma unroll
            for (int q = 0; q < BS; ++q) dst[q] += out[0][q];
            if (nt > 1) {
#pragma unroll
              for (int q = 0; q < BS; ++q) dst[q] += out[1][q];
            }
          }
        } else if (first) {
          uint32_t lo = 0, hi = rlen;
          while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (cols[mid] < col) lo = mid + 1; else hi = mid;
          }
          T *dst = acc + (size_t)lo * BS * BS + l * BS;
          for (int jj = j; jj < CARD; ++jj) {
            if (jj != j && (uint32_t)a.ep[e * a.card + jj] != col) continue;
            T out[2][BS];
            const int nt = Elem::block(a, e, i, jj, l, out);
            if (nt > 0) {
#pragma unroll
              for (int q = 0; q < BS; ++q) dst[q] += out[0][q];
            }
            if (nt > 1) {
#pragma unroll
              for (int q = 0; q < BS; ++q) dst[q] += out[1][q];
            }
          }
        }
      }
      if (Elem::HAS_VEC && gl < BS) {
        T o[4];
        const int nv = Elem::vec(a, e, i, gl, o);
        for (int q = 0; q < nv; ++q) vacc += o[q];
      }
      __syncwarp(gmask);
    }
    if (Elem::HAS_MAT) {
      for (uint32_t q = gl; q < rlen * BS * BS; q += G) {
        const uint32_t pos = q / (BS * BS);
        const int w = q % (BS * BS);
        const bool dg = cols[pos] == (uint32_t)v;
        a.vals[(size_t)r0 * BS * BS + q] = Elem::fin_block(a, (int32_t)v, dg, w / BS, w % BS, acc[q]);
      }
    }
    if (Elem::HAS_VEC && gl < BS) a.f[v * BS + gl] = Elem::fin_vec(a, (int32_t)v, gl, vacc);
    __syncwarp(gmask);
  }
}

// ---------------------------------------------------------------------------
// Element-parallel kernel (one colour of the assembly plan)
// ---------------------------------------------------------------------------
// Each element is computed once: the threads of an element (one per block
// (i, j) for matrix maps, one per local vertex i for vector-only maps) add
// its contributions into the precomputed slots / rows with plain
// read-modify-writes.  No two elements of a colour share a vertex, so no
// other thread touches those values during the launch; colours run in
// order, so every value is summed in the same order on every run.  An
// element that lists one vertex twice sends several blocks to one slot: its
// first thread then adds all of them in turn.  Needs Elem::fin_* to be the
// identity (the outputs start from zero and take the sums as they are).
//
// Sequential form (an element with a repeated vertex, one thread).
template <class Elem, int CARD, int BS, typename T>
__device__ __forceinline__ void colored_row(const AsmArgs<T> &a, int64_t e, int i,
                                            const uint32_t *__restrict__ slots) {
  const int32_t vi = a.ep[e * CARD + i];
  if (Elem::HAS_MAT) {
    for (int j = 0; j < CARD; ++j) {
      const uint32_t sl = slots[(e * CARD + i) * CARD + j];
      if ((int64_t)sl >= a.nnzb) {
        atomicCAS(a.err, 0, 3 /* DEV_SLOT_MISSING */);
        continue;
      }
      for (int l = 0; l < BS; ++l) {
        T out[2][BS];
        const int nt = Elem::block(a, e, i, j, l, out);
        if (nt > 0) {
          T *dst = a.vals + (size_t)sl * BS * BS + l * BS;
          for (int q = 0; q < BS; ++q) {
            T v = dst[q] + out[0][q];
            if (nt > 1) v += out[1][q];
            dst[q] = v;
          }
        }
      }
    }
  }
  if (Elem::HAS_VEC) {
    for (int l = 0; l < BS; ++l) {
      T o[4];
      const int nv = Elem::vec(a, e, i, l, o);
      if (nv > 0) {
        T v = a.f[(int64_t)vi * BS + l];
        for (int q = 0; q < nv; ++q) v += o[q];
        a.f[(int64_t)vi * BS + l] = v;
      }
    }
  }
}

// Usual form (distinct vertices), one thread per block (i, j) of a matrix
// element (its old values loaded first -- independent loads, one memory
// round trip -- then its rows added and stored), and per vertex i for the
// vector part (thread j = 0).  Distinct vertices give distinct slots and
// rows, so nothing aliases.
template <class Elem, int CARD, int BS, typename T>
__device__ __forceinline__ void colored_block(const AsmArgs<T> &a, int64_t e, int i, int j,
                                              const uint32_t *__restrict__ slots) {
  if (Elem::HAS_MAT) {
    const uint32_t sl = slots[(e * CARD + i) * CARD + j];
    if ((int64_t)sl >= a.nnzb) {
      atomicCAS(a.err, 0, 3 /* DEV_SLOT_MISSING */);
    } else {
      T *dst = a.vals + (size_t)sl * BS * BS;
      T old[BS * BS];
#pragma unroll
      for (int q = 0; q < BS * BS; ++q) old[q] = dst[q];
#pragma unroll
      for (int l = 0; l < BS; ++l) {
        T out[2][BS];
        const int nt = Elem::block(a, e, i, j, l, out);
#pragma unroll
        for (int q = 0; q < BS; ++q) {
          if (nt > 0) old[l * BS + q] += out[0][q];
          if (nt > 1) old[l * BS + q] += out[1][q];
        }
      }
#pragma unroll
      for (int q = 0; q < BS * BS; ++q) dst[q] = old[q];
    }
  }
  if (Elem::HAS_VEC && j == 0) {
    const int32_t vi = a.ep[e * CARD + i];
    T fv[BS];
#pragma unroll
    for (int l = 0; l < BS; ++l) fv[l] = a.f[(int64_t)vi * BS + l];
#pragma unroll
    for (int l = 0; l < BS; ++l) {
      T o[4];
      const int nv = Elem::vec(a, e, i, l, o);
      for (int q = 0; q < nv; ++q) fv[l] += o[q];
    }
#pragma unroll
    for (int l = 0; l < BS; ++l) a.f[(int64_t)vi * BS + l] = fv[l];
  }
}

template <class Elem, int CARD, int BS, typename T>
__global__ void __launch_bounds__(256) k_colored(AsmArgs<T> a, const uint32_t *__restrict__ elist,
                                                 int64_t cnt, const uint32_t *__restrict__ slots) {
  constexpr int TPE = Elem::HAS_MAT ? CARD * CARD : CARD;  // threads per element
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < cnt * TPE; t += stride) {
    const int64_t e = elist[t / TPE];
    const int r = (int)(t % TPE);
    const int i = Elem::HAS_MAT ? r / CARD : r, j = Elem::HAS_MAT ? r % CARD : 0;
    const int32_t *vv = a.ep + e * CARD;
    bool rep = false;
#pragma unroll
    for (int i1 = 0; i1 < CARD; ++i1)
#pragma unroll
      for (int i2 = i1 + 1; i2 < CARD; ++i2) rep = rep || vv[i1] == vv[i2];
    if (!rep) {
      colored_block<Elem, CARD, BS, T>(a, e, i, j, slots);
    } else if (r == 0) {
      for (int ii = 0; ii < CARD; ++ii) colored_row<Elem, CARD, BS, T>(a, e, ii, slots);
    }
  }
}

// Elements whose (j, i) block is bitwise the transpose of their (i, j)
// block declare SYM = true; the element-blocks plan then computes and
// stores only the CARD (CARD + 1) / 2 blocks with i <= j, in row order
// (0,0), (0,1), .., (0,CARD-1), (1,1), .., and the slot gather reads the
// transpose for i > j.
template <class E, class = void> struct elem_sym : std::false_type {};
template <class E>
struct elem_sym<E, std::void_t<decltype(E::SYM)>> : std::integral_constant<bool, E::SYM> {};
__device__ __forceinline__ void tri_pair(int C, int r, int &i, int &j) {
  i = 0;
  while (r >= C - i) {
    r -= C - i;
    ++i;
  }
  j = i + r;
}
__device__ __forceinline__ int tri_index(int C, int i, int j) {  // i <= j
  return i * C - i * (i - 1) / 2 + (j - i);
}

// ---------------------------------------------------------------------------
// Element blocks + slot gather (the assembly plan's second form)
// ---------------------------------------------------------------------------
// Phase 1, element-parallel: thread (e, i, j) writes block (i, j) of element
// e (all its terms summed) to eb[(e*CARD + i)*CARD + j] -- consecutive
// threads, consecutive blocks, coalesced -- and for vector maps thread
// (e, i, 0) writes vertex i's contribution to ev[e*CARD + i].  Phase 2:
// every slot sums its contributing blocks (the inverse slot map, sorted by
// block index, i.e. ascending element) and every vertex its contributions
// (its incidence list, ascending element), each written once.  Each element
// is computed once, nothing is read-modified-written, the order of every
// sum is fixed.  Needs Elem::fin_* to be the identity.
// TILE threads per CTA: the element tile is TILE / TPE elements (the
// schedule the assembly tuner picks).
template <class Elem, int CARD, int BS, typename T, int TILE>
__global__ void __launch_bounds__(TILE) k_elem_blocks(AsmArgs<T> a, T *__restrict__ eb,
                                                      T *__restrict__ ev) {
  constexpr bool SY = elem_sym<Elem>::value;
  static_assert(!SY || !Elem::HAS_VEC, "a symmetric element stores blocks only");
  constexpr int TPE = Elem::HAS_MAT ? (SY ? CARD * (CARD + 1) / 2 : CARD * CARD) : CARD;
  // a CTA's TILE consecutive blocks are staged in shared memory and leave in
  // 16-byte stores (the chunk starts TILE * BS*BS * sizeof(T) bytes apart)
  __shared__ __align__(16) T stage[Elem::HAS_MAT ? TILE * BS * BS : 1];
  const int64_t total = a.nE * TPE;
  for (int64_t t0 = (int64_t)blockIdx.x * TILE; t0 < total; t0 += (int64_t)gridDim.x * TILE) {
    const int64_t t = t0 + threadIdx.x;
    if (t < total) {
      const int64_t e = t / TPE;
      const int r = (int)(t % TPE);
      int i = Elem::HAS_MAT ? r / CARD : r, j = Elem::HAS_MAT ? r % CARD : 0;
      if (SY) tri_pair(CARD, r, i, j);
      if (Elem::HAS_MAT) {
#pragma unroll
        for (int l = 0; l < BS; ++l) {
          T out[2][BS];
          const int nt = Elem::block(a, e, i, j, l, out);
#pragma unroll
          for (int q = 0; q < BS; ++q) {
            T v = nt > 0 ? out[0][q] : T(0);
            if (nt > 1) v += out[1][q];
            stage[threadIdx.x * BS * BS + l * BS + q] = v;
          }
        }
      }
      if (Elem::HAS_VEC && j == 0) {
#pragma unroll
        for (int l = 0; l < BS; ++l) {
          T o[4];
          const int nv = Elem::vec(a, e, i, l, o);
          T v = T(0);
          for (int q = 0; q < nv; ++q) v += o[q];
          ev[(e * CARD + i) * BS + l] = v;
        }
      }
    }
    if (Elem::HAS_MAT) {
      __syncthreads();
      const int64_t nval = (min(total, t0 + TILE) - t0) * BS * BS;
      T *dst = eb + t0 * BS * BS;
      constexpr int PER = 16 / sizeof(T);
      if (nval == TILE * BS * BS && (BS * BS * TILE) % PER == 0) {
        const float4 *src4 = reinterpret_cast<const float4 *>(stage);
        float4 *dst4 = reinterpret_cast<float4 *>(dst);
        for (int k = threadIdx.x; k < TILE * BS * BS / PER; k += TILE) dst4[k] = src4[k];
      } else {
        for (int64_t k = threadIdx.x; k < nval; k += TILE) dst[k] = stage[k];
      }
      __syncthreads();
    }
  }
}

// vals[q] = sum of eb blocks src[sptr[q] .. sptr[q+1]); thread per (slot,
// row l); the block indices of up to 8 contributions are loaded before
// their values, and all values before the sum (ascending order kept).
// SC > 0: eb holds only the i <= j blocks of elements of SC endpoints
// (elem_sym); a contribution b = e SC^2 + i SC + j with i > j reads block
// (j, i) transposed.
template <int BS, typename T, int SC = 0>
__global__ void __launch_bounds__(256) k_slot_gather(int64_t nnzb, const uint32_t *__restrict__ sptr,
                                                     const uint32_t *__restrict__ src,
                                                     const T *__restrict__ eb, T *__restrict__ vals) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnzb * BS; t += stride) {
    const int64_t q = t / BS;
    const int l = (int)(t % BS);
    T acc[BS];
#pragma unroll
    for (int m = 0; m < BS; ++m) acc[m] = T(0);
    const uint32_t k1 = sptr[q + 1];
    for (uint32_t k0 = sptr[q]; k0 < k1; k0 += 8) {
      uint32_t b[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) b[u] = k0 + u < k1 ? src[k0 + u] : 0u;
      T x[8][BS];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        size_t blk = b[u];
        bool tr = false;
        if (SC > 0) {
          const uint32_t e = b[u] / (SC * SC), rr = b[u] - e * (SC * SC);
          const int i = (int)rr / SC, j = (int)rr % SC;
          tr = i > j;
          blk = (size_t)e * (SC * (SC + 1) / 2) + tri_index(SC, tr ? j : i, tr ? i : j);
        }
#pragma unroll
        for (int m = 0; m < BS; ++m)
          x[u][m] = k0 + u < k1 ? eb[blk * BS * BS + (tr ? m * BS + l : l * BS + m)] : T(0);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (k0 + u < k1)
#pragma unroll
          for (int m = 0; m < BS; ++m) acc[m] += x[u][m];
    }
#pragma unroll
    for (int m = 0; m < BS; ++m) vals[q * BS * BS + l * BS + m] = acc[m];
  }
}

// f[v] = sum of ev over v's incidences (ascending element); thread per (v, l).
template <int BS, typename T>
__global__ void __launch_bounds__(256) k_vert_gather(int32_t n, const uint32_t *__restrict__ ve_ptr,
                                                     const uint32_t *__restrict__ ve_idx,
                                                     const T *__restrict__ ev, T *__restrict__ f) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)n * BS;
       t += stride) {
    const int64_t v = t / BS;
    const int l = (int)(t % BS);
    T acc = T(0);
    const uint32_t k1 = ve_ptr[v + 1];
    for (uint32_t k = ve_ptr[v]; k < k1; ++k) acc += ev[(size_t)ve_idx[k] * BS + l];
    f[t] = acc;
  }
}

// ---------------------------------------------------------------------------
// Springs (card 2, 3x3 blocks): compute_mass_damping + compute_elasticity of
// apps/springs/isprings.sim:21-68 (form 0) and test/input/program/
// isprings.sim (form 1); MDK = MD + K, f = fmg + fe.
// ---------------------------------------------------------------------------
template <typename T> struct SpringElem {
  static constexpr bool HAS_MAT = true, HAS_VEC = true;
  static constexpr int LANES = 6;
  // the spring's 3x3 k (row l) and fe0 (component l)
  __device__ static void kfe(const AsmArgs<T> &a, int64_t s, int l, T krow[3], T &fe0l) {
    const int32_t e0 = a.ep[2 * s], e1 = a.ep[2 * s + 1];
    const T stiffness = a.k[s];
    T dx[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) dx[q] = a.x[(int64_t)e1 * 3 + q] - a.x[(int64_t)e0 * 3 + q];
    T nrm = 0, nt = 0;
#pragma unroll
    for (int q = 0; q < 3; ++q) nt += dx[q] * dx[q];
    nrm += nt;
    const T L = d_sqrt(nrm);
    const T I3[3] = {T(l == 0), T(l == 1), T(l == 2)};
    if (a.form == 0) {
      T U[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) U[q] = dx[q] / L;
      const T f0 = stiffness * (L - a.l0[s]);
      fe0l = (a.h * f0) * U[l];
      const T s3 = stiffness - (f0 / L), s4 = f0 / L, s5 = a.h * a.h;
#pragma unroll
      for (int q = 0; q < 3; ++q) krow[q] = s5 * ((s3 * (U[l] * U[q])) + (s4 * I3[q]));
    } else {
      const T L0 = a.l0[s];
      const T sc = ((a.h * stiffness) / (L0 * L0)) * (L - L0);
      fe0l = (sc * dx[l]) / L;
      T dxtdx = 0, dt = 0;
#pragma unroll
      for (int q = 0; q < 3; ++q) dt += dx[q] * dx[q];
      dxtdx += dt;
      const T cc = ((a.h * a.h) * stiffness) / (((L0 * L0) * L) * L);
      const T rr = (L - L0) / L;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const T d = dx[l] * dx[q];
        krow[q] = cc * (d + (rr * ((dxtdx * I3[q]) - d)));
      }
    }
  }
  __device__ static int block(const AsmArgs<T> &a, int64_t s, int i, int j, int l,
                             T out[2][3]) {
    const bool f0 = a.fixed[a.ep[2 * s]] != 0, f1 = a.fixed[a.ep[2 * s + 1]] != 0;
    bool write;
    if (!f0 && !f1) write = true;
    else write = (i == j) && ((i == 0) ? !f0 : !f1);
    if (!write) return 0;
    T kr[3], fe;
    kfe(a, s, l, kr, fe);
    const bool neg = (i != j);
#pragma unroll
    for (int q = 0; q < 3; ++q) out[0][q] = neg ? -kr[q] : kr[q];
    return 1;
  }
  __device__ static int vec(const AsmArgs<T> &a, int64_t s, int i, int l, T out[4]) {
    if (a.fixed[a.ep[2 * s + i]]) return 0;
    T kr[3], fe;
    kfe(a, s, l, kr, fe);
    out[0] = (i == 0) ? fe : -fe;
    return 1;
  }
  // MD(p,p): fixed -> only entry (0,0) = 1 (a scalar written to a block);
  // else (mass + h*viscous) * I.  MDK = MD + K (MD is the first operand).
  __device__ static T fin_block(const AsmArgs<T> &a, int32_t p, bool dg, int l, int m, T acc) {
    if (!dg) return acc;
    T md;
    if (a.fixed[p]) md = (l == 0 && m == 0) ? T(1) : T(0);
    else md = (a.m[p] + (a.h * a.viscous)) * T(l == m);
    return md + acc;
  }
  // fmg(p) = mass*v + (h*mass)*grav for free points; f = fmg + fe
  __device__ static T fin_vec(const AsmArgs<T> &a, int32_t p, int l, T acc) {
    T fmg = 0;
    if (!a.fixed[p]) fmg = (a.m[p] * a.v[(int64_t)p * 3 + l]) + ((a.h * a.m[p]) * a.grav[l]);
    return fmg + acc;
  }
};

// ---------------------------------------------------------------------------
// Scalar springs of test/input/program/cg.sim: f gives +-a blocks, eye gives
// I; A = diag*I + scale*K (the lowered matrix expression: diagonal first).
// ---------------------------------------------------------------------------
template <typename T> struct ScalarSpringElem {
  static constexpr bool HAS_MAT = true, HAS_VEC = false;
  static constexpr int LANES = 2;
  __device__ static int block(const AsmArgs<T> &a, int64_t s, int i, int j, int, T out[2][1]) {
    out[0][0] = (i == j) ? a.a[s] : -a.a[s];
    return 1;
  }
  __device__ static int vec(const AsmArgs<T> &, int64_t, int, int, T *) { return 0; }
  __device__ static T fin_block(const AsmArgs<T> &a, int32_t, bool dg, int, int, T acc) {
    return dg ? a.diag + (a.scale * acc) : T(0) + (a.scale * acc);
  }
  __device__ static T fin_vec(const AsmArgs<T> &, int32_t, int, T acc) { return acc; }
};

// ---------------------------------------------------------------------------
// P1 heat (scalar): A_ij = W/20 (1 + δij) + (dt*kappa*W) (g_i . g_j),
// b_i = Σ_j W/20 (1 + δij) T0_j.  g_i = row i of B, g_3 = -(g_0+g_1+g_2).
// ---------------------------------------------------------------------------
template <typename T> struct HeatElem {
  static constexpr bool HAS_MAT = true, HAS_VEC = true;
  static constexpr int LANES = 4;
  __device__ static void grad(const T *Bt, int i, T g[3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      g[d] = (i < 3) ? Bt[i * 3 + d] : -((Bt[0 * 3 + d] + Bt[1 * 3 + d]) + Bt[2 * 3 + d]);
  }
  __device__ static int block(const AsmArgs<T> &a, int64_t t, int i, int j, int, T out[2][1]) {
    const T *Bt = a.B + 9 * t;
    T gi[3], gj[3];
    grad(Bt, i, gi);
    grad(Bt, j, gj);
    const T mw = a.W[t] / T(20.0);
    const T kw = (a.dt * a.kappa[t]) * a.W[t];
    const T mij = (i == j) ? T(2.0) * mw : mw;
    const T gg = (gi[0] * gj[0] + gi[1] * gj[1]) + gi[2] * gj[2];
    out[0][0] = mij + kw * gg;
    return 1;
  }
  __device__ static int vec(const AsmArgs<T> &a, int64_t t, int i, int, T out[4]) {
    const T mw = a.W[t] / T(20.0);
    T bi = 0;
    for (int j = 0; j < 4; ++j) {
      const T mij = (i == j) ? T(2.0) * mw : mw;
      bi += mij * a.T0[a.ep[4 * t + j]];
    }
    out[0] = bi;
    return 1;
  }
  __device__ static T fin_block(const AsmArgs<T> &, int32_t, bool, int, int, T acc) { return acc; }
  __device__ static T fin_vec(const AsmArgs<T> &, int32_t, int, T acc) { return acc; }
};

// Vertex mass of precomputeTetMat: m(v) += (0.25*rho)*W in element order.
template <typename T> struct TetMassElem {
  static constexpr bool HAS_MAT = false, HAS_VEC = true;
  static constexpr int LANES = 1;
  __device__ static int block(const AsmArgs<T> &, int64_t, int, int, int, T (*)[1]) { return 0; }
  __device__ static int vec(const AsmArgs<T> &a, int64_t t, int, int, T out[4]) {
    out[0] = (T(0.25) * a.rho) * a.W[t];
    return 1;
  }
  __device__ static T fin_block(const AsmArgs<T> &, int32_t, bool, int, int, T acc) { return acc; }
  __device__ static T fin_vec(const AsmArgs<T> &, int32_t, int, T acc) { return acc; }
};

// precomputeTetMat (femTet.sim, apps/fem/fem_linear.sim:176-193), per tet:
// Ds(jj,ii) = x_ii(jj) - x_3(jj); B = inv(Ds); W = -(1/6) det(Ds).
template <typename T>
__global__ void k_tet_precompute(int64_t nT, const int32_t *__restrict__ tets,
                                 const T *__restrict__ x, T *__restrict__ B, T *__restrict__ W) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nT;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t *v = tets + 4 * t;
    T M[9], Bi[9];
#pragma unroll
    for (int ii = 0; ii < 3; ++ii)
#pragma unroll
      for (int jj = 0; jj < 3; ++jj)
        M[jj * 3 + ii] = x[(int64_t)v[ii] * 3 + jj] - x[(int64_t)v[3] * 3 + jj];
    d_inv3(M, Bi);
#pragma unroll
    for (int q = 0; q < 9; ++q) B[t * 9 + q] = T(1.0) * Bi[q];
    W[t] = -(T(1.0) / T(6.0)) * d_det3(M);
  }
}


// ---------------------------------------------------------------------------
// Tetrahedra (card 4, 3x3 blocks): test/input/program/femTet.sim (neo-Hookean)
// and apps/fem/fem_linear.sim (linear).  Constraint c(v) > 0 removes the
// vertex's couplings; the lumped element mass m*I = 0.25*rho*W*I is added to
// every vertex's diagonal block after the stiffness part of the element.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void tet_F(const AsmArgs<T> &a, int64_t t, T F[9]) {
  const int32_t *v = a.ep + 4 * t;
  T Ds[9];
#pragma unroll
  for (int ii = 0; ii < 3; ++ii)
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
      Ds[jj * 3 + ii] = a.x[(int64_t)v[ii] * 3 + jj] - a.x[(int64_t)v[3] * 3 + jj];
  d_mm3(Ds, a.B + 9 * t, F);
}

// H = ((-W) * P) * B'
template <typename T>
__device__ __forceinline__ void tet_H(T W, const T *P, const T *B, T *H) {
  T s[9], Bt[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) s[q] = (-W) * P[q];
  d_tr3(B, Bt);
  d_mm3(s, Bt, H);
}

// Element blocks of the neo-Hookean tangent (femTet.sim compute_stiffness):
// eb[(t*16 + jj*4 + row)*9 + a*3 + b] = -(h*h*Kb_row(jj, a, b)) when both
// vertices are free, else 0.  One thread per tet.  dPdF is evaluated exactly
// as the .sim writes it, with log(det F) and inv(F) computed once per tet
// (they are the same values for all twelve calls).
template <typename T>
__global__ void k_neo_blocks(AsmArgs<T> a) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < a.nE;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t *vv = a.ep + 4 * t;
    const T *Bt = a.B + 9 * t;
    const T u = a.mu[t], l = a.lam[t], W = a.W[t];
    T F[9];
    tet_F(a, t, F);
    const T JJ = d_log(d_det3(F));
    T Finv[9], FinvT[9], Btr[9];
    d_inv3(F, Finv);
    d_tr3(Finv, FinvT);
    d_tr3(Bt, Btr);
    const T cc = u - l * JJ;
    bool freev[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) freev[q] = a.c[vv[q]] <= 0;
    T *out = const_cast<T *>(a.eb) + (size_t)t * 144;
    for (int row = 0; row < 4; ++row) {
      T dFRow[3];
#pragma unroll
      for (int ll = 0; ll < 3; ++ll)
        dFRow[ll] = (row < 3) ? Bt[row * 3 + ll]
                              : -((Bt[0 * 3 + ll] + Bt[1 * 3 + ll]) + Bt[2 * 3 + ll]);
      T Kb[36];
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) {
        T dF[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) dF[q] = T(0);
#pragma unroll
        for (int ll = 0; ll < 3; ++ll) dF[kk * 3 + ll] = dFRow[ll];
        T FidF[9], FidFT[9], s1[9], t2[9], dP[9], dH[9], sW[9];
        d_mm3(Finv, dF, FidF);
        d_tr3(FidF, FidFT);
#pragma unroll
        for (int q = 0; q < 9; ++q) s1[q] = cc * FinvT[q];
        d_mm3(s1, FidFT, t2);
        const T trc = FidF[0] + FidF[4] + FidF[8];
        const T c3 = l * trc;
#pragma unroll
        for (int q = 0; q < 9; ++q) dP[q] = ((u * dF[q]) + t2[q]) + (c3 * FinvT[q]);
#pragma unroll
        for (int q = 0; q < 9; ++q) sW[q] = (-W) * dP[q];
        d_mm3(sW, Btr, dH);
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) {
#pragma unroll
          for (int ll = 0; ll < 3; ++ll) Kb[ii * 9 + ll * 3 + kk] = dH[ll * 3 + ii];
          Kb[3 * 9 + ii * 3 + kk] = -((dH[ii * 3 + 0] + dH[ii * 3 + 1]) + dH[ii * 3 + 2]);
        }
      }
      const T hh = a.h * a.h;
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const bool w = freev[jj] && freev[row];
#pragma unroll
        for (int q = 0; q < 9; ++q) out[(jj * 4 + row) * 9 + q] = w ? -(hh * Kb[jj * 9 + q]) : T(0);
      }
    }
  }
}

// Generic `map f to E reduce +` with the element function already evaluated
// by the caller: block (i, j) of element e is eb[((e*CARD + i)*CARD + j)*BS*BS
// + l*BS + m] (src/lower/lower_maps.cpp:54-128 lowers `A(p(i),p(j)) = blk`
// to `+=` of blk into the slot of (p(i), p(j)); blocks f does not write are
// zero).  The row owners add them in element order, as the reference's loop.
template <typename T, int BS, int CARD> struct BlocksElem {
  static constexpr bool HAS_MAT = true, HAS_VEC = false;
  static constexpr int LANES = CARD * BS;
  __device__ static int block(const AsmArgs<T> &a, int64_t e, int i, int j, int l,
                              T out[2][BS]) {
    const T *b = a.eb + (((size_t)e * CARD + i) * CARD + j) * BS * BS + l * BS;
#pragma unroll
    for (int q = 0; q < BS; ++q) out[0][q] = b[q];
    return 1;
  }
  __device__ static int vec(const AsmArgs<T> &, int64_t, int, int, T *) { return 0; }
  __device__ static T fin_block(const AsmArgs<T> &, int32_t, bool, int, int, T acc) { return acc; }
  __device__ static T fin_vec(const AsmArgs<T> &, int32_t, int, T acc) { return acc; }
};

// Row owner over element blocks: block (i, j) of tet e from eb, then m*I on
// the diagonal (the element's second write to K(v(i), v(i))).
template <typename T> struct EbGatherElem {
  static constexpr bool HAS_MAT = true, HAS_VEC = false;
  static constexpr int LANES = 12;
  __device__ static int block(const AsmArgs<T> &a, int64_t t, int i, int j, int l, T out[2][3]) {
    const T *b = a.eb + ((size_t)t * 16 + i * 4 + j) * 9 + l * 3;
#pragma unroll
    for (int q = 0; q < 3; ++q) out[0][q] = b[q];
    if (i != j) return 1;
    const T m = (T(0.25) * a.rho) * a.W[t];
#pragma unroll
    for (int q = 0; q < 3; ++q) out[1][q] = m * T(l == q);
    return 2;
  }
  __device__ static int vec(const AsmArgs<T> &, int64_t, int, int, T *) { return 0; }
  __device__ static T fin_block(const AsmArgs<T> &, int32_t, bool, int, int, T acc) { return acc; }
  __device__ static T fin_vec(const AsmArgs<T> &, int32_t, int, T acc) { return acc; }
};

// fem_linear.sim:105-174: Ke = ((W * Bm') * E) * Bm with Voigt E and the
// strain-displacement Bm built from dN, in that operation order (EXACT), or
// the algebraically equal closed form (fast):
//   K_ij[a][b] = W (lam g_ia g_jb + mu g_ib g_ja + mu (g_i . g_j) δab).
// K(v(i), v(j)) += h*h*K_ij when both vertices are free; then m*I on (i, i).
template <typename T, bool EXACT> struct LinTetElem {
  static constexpr bool HAS_MAT = true, HAS_VEC = false;
  // the fast form's (j, i) block is bitwise the transpose of (i, j)
  static constexpr bool SYM = !EXACT;
  static constexpr int LANES = 12;
  __device__ static void dN(const T *Bt, int vi, T g[3]) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (vi < 3) g[d] = Bt[vi * 3 + d];
      else g[d] = ((T(0) - Bt[0 * 3 + d]) - Bt[1 * 3 + d]) - Bt[2 * 3 + d];
    }
  }
  // column r (0..11) of Bm: 6 entries
  __device__ static void bm_col(const T *Bt, int r, T col[6]) {
    const int vi = r / 3, di = r % 3;
    T g[3];
    dN(Bt, vi, g);
#pragma unroll
    for (int k = 0; k < 6; ++k) col[k] = T(0);
    col[di] = g[di];
    if (di == 0) { col[3] = g[1]; col[5] = g[2]; }
    if (di == 1) { col[3] = g[0]; col[4] = g[2]; }
    if (di == 2) { col[4] = g[1]; col[5] = g[0]; }
  }
  __device__ static int block(const AsmArgs<T> &a, int64_t t, int i, int j, int l, T out[2][3]) {
    const int32_t *vv = a.ep + 4 * t;
    const bool both = a.c[vv[i]] <= 0 && a.c[vv[j]] <= 0;
    const T *Bt = a.B + 9 * t;
    const T W = a.W[t], u = a.mu[t], lm = a.lam[t];
    T k3[3] = {T(0), T(0), T(0)};
    if (both) {
      if (EXACT) {
        // E(c, a): l off-diagonal in the 3x3 normal part, l+2u on it, u shear
        T cr[6];
        bm_col(Bt, 3 * i + l, cr);
        T Trow[6];
#pragma unroll
        for (int ac = 0; ac < 6; ++ac) {
          T s = 0;
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            T Eka;
            if (k < 3 && ac < 3) Eka = (k == ac) ? lm + T(2.0) * u : lm;
            else Eka = (k == ac) ? u : T(0);
            s += (W * cr[k]) * Eka;
          }
          Trow[ac] = s;
        }
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          T cc[6];
          bm_col(Bt, 3 * j + m, cc);
          T s = 0;
#pragma unroll
          for (int k = 0; k < 6; ++k) s += Trow[k] * cc[k];
          k3[m] = (a.h * a.h) * s;
        }
      } else {
        // Every product pairs one factor of vertex i with one of vertex j and
        // no operation is contracted, so the (j, i) block is bitwise the
        // transpose of the (i, j) block and the assembled matrix is exactly
        // symmetric (the symmetric-storage SpMV reads only its upper half).
        T gi[3], gj[3];
        dN(Bt, i, gi);
        dN(Bt, j, gj);
        const T gij =
            add_rn(add_rn(mul_rn(gi[0], gj[0]), mul_rn(gi[1], gj[1])), mul_rn(gi[2], gj[2]));
        const T hw = mul_rn(mul_rn(a.h, a.h), W);
        const T ug = mul_rn(u, gij);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          T t = add_rn(mul_rn(lm, mul_rn(gi[l], gj[m])), mul_rn(u, mul_rn(gi[m], gj[l])));
          if (l == m) t = add_rn(t, ug);
          k3[m] = mul_rn(hw, t);
        }
      }
    }
    int nt = 0;
    if (both) {
#pragma unroll
      for (int m = 0; m < 3; ++m) out[0][m] = k3[m];
      nt = 1;
    }
    if (i == j) {
      const T mm = (T(0.25) * a.rho) * W;
#pragma unroll
      for (int m = 0; m < 3; ++m) out[nt][m] = mm * T(l == m);
      ++nt;
    }
    return nt;
  }
  __device__ static int vec(const AsmArgs<T> &, int64_t, int, int, T *) { return 0; }
  __device__ static T fin_block(const AsmArgs<T> &, int32_t, bool, int, int, T acc) { return acc; }
  __device__ static T fin_vec(const AsmArgs<T> &, int32_t, int, T acc) { return acc; }
};

// compute_force of femTet.sim (NEO) / fem_linear.sim:55-93 (linear), vector
// only.  Local vertex i < 3 receives h*H(:,i); vertex 3 receives -h*H(:,ii)
// for ii = 0, 1, 2 in turn; then every free vertex receives h*fg + m*v.
template <typename T, bool NEO> struct TetForceElem {
  static constexpr bool HAS_MAT = false, HAS_VEC = true;
  static constexpr int LANES = 3;
  __device__ static int block(const AsmArgs<T> &, int64_t, int, int, int, T (*)[3]) { return 0; }
  __device__ static int vec(const AsmArgs<T> &a, int64_t t, int i, int l, T out[4]) {
    const int32_t *vv = a.ep + 4 * t;
    if (a.c[vv[i]] > 0) return 0;
    const T *Bt = a.B + 9 * t;
    const T u = a.mu[t], lm = a.lam[t], W = a.W[t];
    T F[9], P[9], H[9];
    tet_F(a, t, F);
    if (NEO) {
      const T JJ = d_log(d_det3(F));
      T Fi[9], FinvT[9];
      d_inv3(F, Fi);
      d_tr3(Fi, FinvT);
#pragma unroll
      for (int q = 0; q < 9; ++q) P[q] = (u * (F[q] - FinvT[q])) + ((lm * JJ) * FinvT[q]);
    } else {
      T FI[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) FI[q] = F[q] - T((q % 4) == 0);
      const T tr = (FI[0] + FI[4]) + FI[8];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int s2 = 0; s2 < 3; ++s2)
          P[r * 3 + s2] = (u * (FI[r * 3 + s2] + FI[s2 * 3 + r])) + ((lm * tr) * T(r == s2));
    }
    tet_H(W, P, Bt, H);
    int nt = 0;
    if (i < 3) {
      out[nt++] = a.h * H[l * 3 + i];
    } else {
#pragma unroll
      for (int ii = 0; ii < 3; ++ii) out[nt++] = (-a.h) * H[l * 3 + ii];
    }
    const T m = (T(0.25) * a.rho) * W;
    const T fg = m * a.grav[l];
    out[nt++] = (a.h * fg) + (m * a.v[(int64_t)vv[i] * 3 + l]);
    return nt;
  }
  __device__ static T fin_block(const AsmArgs<T> &, int32_t, bool, int, int, T acc) { return acc; }
  __device__ static T fin_vec(const AsmArgs<T> &, int32_t, int, T acc) { return acc; }
};

}  // namespace sg
