// Element kernels compiled at run time: the caller gives the element
// function of a `map f to E reduce +` as CUDA C++ source, and NVRTC compiles
// it together with a row-owner assembly kernel for sm_103a.  This is the
// code-generation end of the reference's map lowering (src/inline.cpp:
// 690-888 inlines the element function into the element loop,
// src/lower/lower_maps.cpp:54-128 turns its writes into `+=` on the slots)
// with the element function written directly in CUDA instead of produced
// from a .sim program by the reference's frontend.
//
// The element function's contract (real is float or double, BS and CARD are
// the block size and the endpoints per element, sg_block is real[BS][BS]):
//
//   __device__ int element_block(long long e, int i, int j, const int *ep,
//                                const real *const *f, sg_block *blk);
//
// it writes the terms that element e adds to block (i, j) (ep: its CARD
// endpoints; f: the caller's field arrays) into blk[0], blk[1] and returns
// how many there are (0 .. SG_TERMS = 2).  Each term is a separate `+=` on
// the slot, as each write of the reference's element function is after
// lowering (a diagonal block that receives a stiffness and a mass write gets
// two adds).  The generated kernel is the row-owner form of the hand-written
// ones: a warp owns block row v; its lanes compute the blocks of 32 / CARD
// incidences of v at once (lane = k * CARD + j); then, incidence by
// incidence in ascending element order, the lanes of (j, block row) add the
// terms into a shared-memory image of the row, so every slot sums its
// contributions from zero in the reference's order (ascending element, then
// ascending j, then term).  An element that lists a vertex twice sends
// several j to one slot: the first such j adds them all in ascending j.
//
// NVRTC is loaded with dlopen at the first use and the image is loaded
// through the runtime's library API, so the library itself links neither.
#include <dlfcn.h>
#include <nvrtc.h>
#include <stdint.h>

#include <string.h>

#include <string>
#include <vector>

#include "sg_internal.cuh"

namespace sg {
namespace {

struct Nvrtc {
  bool tried = false, ok = false;
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

Nvrtc load_nvrtc() {
  Nvrtc N;
  N.tried = true;
  void *h = dlopen("libnvrtc.so.13", RTLD_NOW | RTLD_LOCAL);
  if (!h) h = dlopen("libnvrtc.so", RTLD_NOW | RTLD_LOCAL);
  if (!h) return N;
  N.create = (decltype(N.create))dlsym(h, "nvrtcCreateProgram");
  N.compile = (decltype(N.compile))dlsym(h, "nvrtcCompileProgram");
  N.log_size = (decltype(N.log_size))dlsym(h, "nvrtcGetProgramLogSize");
  N.log = (decltype(N.log))dlsym(h, "nvrtcGetProgramLog");
  N.cubin_size = (decltype(N.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
  N.cubin = (decltype(N.cubin))dlsym(h, "nvrtcGetCUBIN");
  N.destroy = (decltype(N.destroy))dlsym(h, "nvrtcDestroyProgram");
  N.ok = N.create && N.compile && N.log_size && N.log && N.cubin_size && N.cubin && N.destroy;
  return N;
}

// Loaded once per process; the static's initialisation is thread-safe, and
// NVRTC programs may be compiled from several threads at once.
const Nvrtc &nvrtc() {
  static const Nvrtc N = load_nvrtc();
  return N;
}

constexpr int JIT_MAX_FIELDS = 8;
constexpr int JIT_WARPS = 4;
constexpr int JIT_TERMS = 2;  // SG_TERMS of the generated source

// The generated kernel around the caller's element function.
const char *kJitPrologue = R"(
typedef SG_REAL real;
typedef real sg_block[BS][BS];
#define SG_TERMS 2
)";

const char *kJitKernel = R"(
struct SgFields { const real *p[8]; };
extern "C" __global__ void __launch_bounds__(128)
sg_jit_rows(int n, const unsigned *__restrict__ ve_ptr, const unsigned *__restrict__ ve_idx,
            const int *__restrict__ ep_all, const unsigned *__restrict__ rowptr,
            const unsigned *__restrict__ colidx, int maxrow, SgFields f,
            real *__restrict__ vals, int *err) {
  constexpr int BB = BS * BS, KI = 32 / CARD, NS = KI * CARD;
  extern __shared__ __align__(16) unsigned char sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  // per warp: acc[maxrow*BB], stage[NS*SG_TERMS*BB] (reals), then cols[maxrow],
  // slot[NS], nts[NS], colk[NS] (ints); each kind laid out warp after warp
  real *acc = reinterpret_cast<real *>(sm) + (size_t)warp * maxrow * BB;
  real *stage = reinterpret_cast<real *>(sm) + (size_t)nwarp * maxrow * BB +
                (size_t)warp * NS * SG_TERMS * BB;
  unsigned *ibase = reinterpret_cast<unsigned *>(reinterpret_cast<real *>(sm) +
                                                 (size_t)nwarp * (maxrow * BB + NS * SG_TERMS * BB));
  unsigned *cols = ibase + (size_t)warp * maxrow;
  int *slot = reinterpret_cast<int *>(ibase + (size_t)nwarp * maxrow) + (size_t)warp * 3 * NS;
  int *nts = slot + NS;
  unsigned *colk = reinterpret_cast<unsigned *>(nts + NS);
  for (long long v = (long long)blockIdx.x * nwarp + warp; v < n;
       v += (long long)gridDim.x * nwarp) {
    const unsigned r0 = rowptr[v], rlen = rowptr[v + 1] - r0;
    if ((int)rlen > maxrow) {
      if (lane == 0) atomicCAS(err, 0, 4);
      continue;
    }
    for (unsigned q = lane; q < rlen; q += 32) cols[q] = colidx[r0 + q];
    for (unsigned q = lane; q < rlen * BB; q += 32) acc[q] = real(0);
    __syncwarp();
    const unsigned iend = ve_ptr[v + 1];
    for (unsigned it0 = ve_ptr[v]; it0 < iend; it0 += KI) {
      const int kn = (int)((iend - it0) < (unsigned)KI ? (iend - it0) : (unsigned)KI);
      const int k = lane / CARD, j = lane - k * CARD;
      if (k < kn) {
        const unsigned t = ve_idx[it0 + k];
        const long long e = t / CARD;
        const int i = (int)(t - (unsigned)e * CARD);
        const int *ep = ep_all + e * CARD;
        sg_block blk[SG_TERMS];
        for (int q = 0; q < SG_TERMS; ++q)
          for (int a = 0; a < BS; ++a)
            for (int b = 0; b < BS; ++b) blk[q][a][b] = real(0);
        int nt = element_block(e, i, j, ep, f.p, blk);
        nt = nt < 0 ? 0 : (nt > SG_TERMS ? SG_TERMS : nt);
        for (int q = 0; q < nt; ++q)
          for (int a = 0; a < BS; ++a)
            for (int b = 0; b < BS; ++b) stage[((lane * SG_TERMS + q) * BS + a) * BS + b] = blk[q][a][b];
        const unsigned col = (unsigned)ep[j];
        unsigned lo = 0, hi = rlen;
        while (lo < hi) {
          const unsigned mid = (lo + hi) >> 1;
          if (cols[mid] < col) lo = mid + 1;
          else hi = mid;
        }
        int s = (int)lo;
        if (lo >= rlen || cols[lo] != col) {
          if (nt > 0) atomicCAS(err, 0, 3);
          s = -1;
        }
        slot[lane] = s;
        nts[lane] = nt;
        colk[lane] = col;
      }
      __syncwarp();
      for (int kk = 0; kk < kn; ++kk) {
        for (int w = lane; w < CARD * BS; w += 32) {
          const int jw = w / BS, a = w - jw * BS, base = kk * CARD;
          const unsigned col = colk[base + jw];
          bool first = true;
          for (int j2 = 0; j2 < jw; ++j2) first = first && colk[base + j2] != col;
          const int s = slot[base + jw];
          if (!first || s < 0) continue;
          real *dst = acc + (size_t)s * BB + a * BS;
          for (int jj = jw; jj < CARD; ++jj) {
            if (colk[base + jj] != col) continue;
            const real *src = stage + (size_t)(base + jj) * SG_TERMS * BB + a * BS;
            for (int q = 0; q < nts[base + jj]; ++q)
              for (int b = 0; b < BS; ++b) dst[b] += src[q * BB + b];
          }
        }
        __syncwarp();
      }
    }
    for (unsigned q = lane; q < rlen * BB; q += 32) vals[(size_t)r0 * BB + q] = acc[q];
    __syncwarp();
  }
}
)";

// The generated kernel around a vector element function (the result of a
// `map f to E reduce +` that is a system vector):
//   __device__ int element_vector(long long e, int i, const int *ep,
//                                 const real *const *f, sg_vec *vec);
// writes the terms element e adds to its endpoint i (sg_vec = real[BS], at
// most SG_VTERMS) and returns their count.  A thread owns a vertex and adds,
// from zero, its incidences' terms in ascending (element, local index),
// each element's terms in the order it returns them -- the lowered map's
// order, in which each write `f(v(i)) = x` is one `+=` on the vertex.
const char *kJitVecKernel = R"(
struct SgFields { const real *p[8]; };
extern "C" __global__ void __launch_bounds__(128)
sg_jit_vec(int n, const unsigned *__restrict__ ve_ptr, const unsigned *__restrict__ ve_idx,
           const int *__restrict__ ep_all, SgFields f, real *__restrict__ vals) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n;
       v += (long long)gridDim.x * blockDim.x) {
    real acc[BS];
    for (int a = 0; a < BS; ++a) acc[a] = real(0);
    const unsigned iend = ve_ptr[v + 1];
    for (unsigned it = ve_ptr[v]; it < iend; ++it) {
      const unsigned t = ve_idx[it];
      const long long e = t / CARD;
      const int i = (int)(t - (unsigned)e * CARD);
      sg_vec terms[SG_VTERMS];
      for (int q = 0; q < SG_VTERMS; ++q)
        for (int a = 0; a < BS; ++a) terms[q][a] = real(0);
      int nt = element_vector(e, i, ep_all + e * CARD, f.p, terms);
      nt = nt < 0 ? 0 : (nt > SG_VTERMS ? SG_VTERMS : nt);
      for (int q = 0; q < nt; ++q)
        for (int a = 0; a < BS; ++a) acc[a] += terms[q][a];
    }
    for (int a = 0; a < BS; ++a) vals[(size_t)v * BS + a] = acc[a];
  }
}
)";

struct JitAssembly {
  Ctx *c = nullptr;
  int card = 0, bs = 0, dtype = 0;
  bool vec = false;
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
};

struct JitFields {
  const void *p[JIT_MAX_FIELDS];
};

}  // namespace
}  // namespace sg

using namespace sg;

namespace {

// Compiles the generated source; on success `image` holds the CUBIN, on a
// compile error `log` the compiler's log and the result is SG_ERR_ARG.
int jit_compile(const char *element_src, int32_t card, int32_t bs, int dtype, int32_t exact,
                std::vector<char> &image, std::string &log, bool vec = false) {
  SG_REQUIRE(element_src, "sg_jit: null source");
  SG_REQUIRE(card >= 1 && card <= 32 && bs >= 1 && bs <= 16,
             "sg_jit: card %d bs %d (card 1..32, bs 1..16)", card, bs);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_jit: dtype %d", dtype);
  const Nvrtc &N = nvrtc();
  if (!N.ok) return set_error(SG_ERR_UNSUPPORTED, "sg_jit: NVRTC not found");
  std::string src = "#define SG_REAL " + std::string(dtype == SG_F64 ? "double" : "float") +
                    "\n#define BS " + std::to_string(bs) + "\n#define CARD " +
                    std::to_string(card) + "\n" + kJitPrologue +
                    (vec ? "typedef real sg_vec[BS];\n#define SG_VTERMS 8\n" : "") + "\n" +
                    element_src + "\n" + (vec ? kJitVecKernel : kJitKernel);
  nvrtcProgram prog = nullptr;
  if (N.create(&prog, src.c_str(), "sg_jit_element.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
    return set_error(SG_ERR_UNSUPPORTED, "sg_jit: nvrtcCreateProgram failed");
  std::vector<const char *> opts = {"-arch=sm_103a", "-std=c++17",
                                    exact ? "--fmad=false" : "--fmad=true"};
  const nvrtcResult rc = N.compile(prog, (int)opts.size(), opts.data());
  size_t ls = 0;
  N.log_size(prog, &ls);
  log.assign(ls, '\0');
  if (ls) N.log(prog, &log[0]);
  if (!log.empty() && log.back() == '\0') log.pop_back();
  if (rc != NVRTC_SUCCESS) {
    N.destroy(&prog);
    std::string shown = log.size() > 1500 ? log.substr(0, 1500) : log;
    return set_error(SG_ERR_ARG, "sg_jit: the element source does not compile:\n%s",
                     shown.c_str());
  }
  size_t cs = 0;
  N.cubin_size(prog, &cs);
  image.resize(cs);
  N.cubin(prog, image.data());
  N.destroy(&prog);
  return SG_OK;
}

}  // namespace

extern "C" {

int sg_jit_check_source(const char *element_src, int32_t card, int32_t bs, int dtype,
                        int32_t exact, char *log, int64_t log_cap) {
  std::vector<char> image;
  std::string lg;
  const int rc = jit_compile(element_src, card, bs, dtype, exact, image, lg);
  if (log && log_cap > 0) {
    const size_t k = lg.size() < (size_t)(log_cap - 1) ? lg.size() : (size_t)(log_cap - 1);
    memcpy(log, lg.data(), k);
    log[k] = '\0';
  }
  return rc;
}

int sg_jit_check_vector_source(const char *element_src, int32_t card, int32_t bs, int dtype,
                               int32_t exact, char *log, int64_t log_cap) {
  std::vector<char> image;
  std::string lg;
  const int rc = jit_compile(element_src, card, bs, dtype, exact, image, lg, true);
  if (log && log_cap > 0) {
    const size_t k = lg.size() < (size_t)(log_cap - 1) ? lg.size() : (size_t)(log_cap - 1);
    memcpy(log, lg.data(), k);
    log[k] = '\0';
  }
  return rc;
}

static int jit_create(sg_ctx *h, const char *element_src, int32_t card, int32_t bs, int dtype,
                      int32_t exact, bool vec, sg_jit_assembly **out) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && element_src && out, "sg_jit: null argument");
  std::vector<char> image;
  std::string log;
  const int rc = jit_compile(element_src, card, bs, dtype, exact, image, log, vec);
  if (rc != SG_OK) return rc;
  auto *J = new JitAssembly();
  J->c = c;
  J->card = card;
  J->bs = bs;
  J->dtype = dtype;
  J->vec = vec;
  cudaError_t e = cudaLibraryLoadData(&J->lib, image.data(), nullptr, nullptr, 0, nullptr,
                                      nullptr, 0);
  if (e == cudaSuccess)
    e = cudaLibraryGetKernel(&J->kernel, J->lib, vec ? "sg_jit_vec" : "sg_jit_rows");
  if (e != cudaSuccess) {
    if (J->lib) cudaLibraryUnload(J->lib);
    delete J;
    return set_error(SG_ERR_CUDA, "sg_jit: %s", cudaGetErrorString(e));
  }
  ctx_retain(c);
  *out = reinterpret_cast<sg_jit_assembly *>(J);
  return SG_OK;
}

int sg_jit_assembly_create(sg_ctx *h, const char *element_src, int32_t card, int32_t bs,
                           int dtype, int32_t exact, sg_jit_assembly **out) {
  return jit_create(h, element_src, card, bs, dtype, exact, false, out);
}

int sg_jit_vector_create(sg_ctx *h, const char *element_src, int32_t card, int32_t bs,
                         int dtype, int32_t exact, sg_jit_assembly **out) {
  return jit_create(h, element_src, card, bs, dtype, exact, true, out);
}

int sg_jit_assemble_vector(sg_jit_assembly *hj, const sg_mesh *m, const void *const *h_fields,
                           int32_t nfields, void *vals) {
  JitAssembly *J = reinterpret_cast<JitAssembly *>(hj);
  DeviceGuard dg_(J ? J->c : nullptr);
  SG_REQUIRE(J && m && vals, "sg_jit_assemble_vector: null argument");
  SG_REQUIRE(J->vec, "sg_jit_assemble_vector: the handle holds a matrix element function");
  SG_REQUIRE(m->card == J->card, "sg_jit_assemble_vector: mesh card %d, kernel card %d",
             m->card, J->card);
  SG_REQUIRE(nfields >= 0 && nfields <= JIT_MAX_FIELDS && (nfields == 0 || h_fields),
             "sg_jit_assemble_vector: %d fields (at most %d)", nfields, JIT_MAX_FIELDS);
  SG_REQUIRE(m->ve_ptr && (m->nE == 0 || (m->ve_idx && m->endpoints)),
             "sg_jit_assemble_vector: mesh incidence missing");
  if (m->n == 0) return SG_OK;
  Ctx *c = J->c;
  JitFields f{};
  for (int k = 0; k < nfields; ++k) f.p[k] = h_fields[k];
  int n = m->n;
  const unsigned *ve_ptr = m->ve_ptr, *ve_idx = m->ve_idx;
  const int *ep = m->endpoints;
  void *args[] = {&n, &ve_ptr, &ve_idx, &ep, &f, &vals};
  const int grid = grid_for(c, (int64_t)m->n, 128, 8);
  SG_CHECK_CUDA(cudaLaunchKernel((const void *)J->kernel, dim3(grid), dim3(128), args, 0,
                                 c->stream));
  return SG_OK;
}

int sg_jit_assemble(sg_jit_assembly *hj, const sg_mesh *m, const void *const *h_fields,
                    int32_t nfields, void *vals) {
  JitAssembly *J = reinterpret_cast<JitAssembly *>(hj);
  DeviceGuard dg_(J ? J->c : nullptr);
  SG_REQUIRE(J && m && vals, "sg_jit_assemble: null argument");
  SG_REQUIRE(!J->vec, "sg_jit_assemble: the handle holds a vector element function");
  SG_REQUIRE(m->card == J->card, "sg_jit_assemble: mesh card %d, kernel card %d", m->card,
             J->card);
  SG_REQUIRE(nfields >= 0 && nfields <= JIT_MAX_FIELDS && (nfields == 0 || h_fields),
             "sg_jit_assemble: %d fields (at most %d)", nfields, JIT_MAX_FIELDS);
  SG_REQUIRE(m->rowptr && m->colidx && m->ve_ptr && (m->nE == 0 || (m->ve_idx && m->endpoints)),
             "sg_jit_assemble: mesh arrays missing");
  if (m->n == 0) return SG_OK;
  Ctx *c = J->c;
  const size_t rs = J->dtype == SG_F64 ? 8 : 4;
  const int maxrow = m->maxrow > 0 ? m->maxrow : 1;
  const size_t bb = (size_t)J->bs * J->bs, ns = (size_t)(32 / J->card) * J->card;
  const size_t per_warp = maxrow * bb * rs + ns * JIT_TERMS * bb * rs + maxrow * 4 + 3 * ns * 4;
  int warps = JIT_WARPS;
  while (warps > 1 && warps * per_warp > 48 * 1024) warps >>= 1;
  const size_t sh = warps * per_warp;
  if (sh > 48 * 1024)
    return set_error(SG_ERR_UNSUPPORTED, "sg_jit_assemble: a row of %d blocks exceeds shared memory",
                     maxrow);
  JitFields f{};
  for (int k = 0; k < nfields; ++k) f.p[k] = h_fields[k];
  int n = m->n;
  const unsigned *ve_ptr = m->ve_ptr, *ve_idx = m->ve_idx, *rowptr = m->rowptr,
                 *colidx = m->colidx;
  const int *ep = m->endpoints;
  int mr = maxrow;
  int *err = c->d_err;
  void *args[] = {&n, &ve_ptr, &ve_idx, &ep, &rowptr, &colidx, &mr, &f, &vals, &err};
  const int grid = grid_for(c, (int64_t)m->n * 32, warps * 32, 32 / warps * 2);
  SG_CHECK_CUDA(cudaLaunchKernel((const void *)J->kernel, dim3(grid), dim3(warps * 32), args,
                                 sh, c->stream));
  return SG_OK;
}

int sg_jit_assembly_destroy(sg_jit_assembly *hj) {
  JitAssembly *J = reinterpret_cast<JitAssembly *>(hj);
  DeviceGuard dg_(J ? J->c : nullptr);
  if (!J) return SG_OK;
  cudaStreamSynchronize(J->c->stream);
  if (J->lib) cudaLibraryUnload(J->lib);
  Ctx *c = J->c;
  delete J;
  ctx_release(c);
  return SG_OK;
}

}  // extern "C"
