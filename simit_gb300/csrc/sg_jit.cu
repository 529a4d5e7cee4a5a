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
// the block size and the endpoints per element):
//
//   __device__ int element_block(long long e, int i, int j, const int *ep,
//                                const real *const *f, real blk[BS][BS]);
//
// it writes block (i, j) of element e (ep: its CARD endpoints; f: the
// caller's field arrays) and returns 0 when the element writes nothing
// there.  The generated kernel is the row-owner form of the hand-written
// ones: a warp owns block row v, walks its incidences in ascending element
// order, lane j computes block (i, j), and lanes add the blocks into a
// shared-memory image of the row in ascending j, so every slot sums its
// contributions in the reference's order from zero.
//
// NVRTC is loaded with dlopen at the first use and the image is loaded
// through the runtime's library API, so the library itself links neither.
#include <dlfcn.h>
#include <nvrtc.h>
#include <stdint.h>

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

Nvrtc &nvrtc() {
  static Nvrtc N;
  if (N.tried) return N;
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

constexpr int JIT_MAX_FIELDS = 8;
constexpr int JIT_WARPS = 4;

// The generated kernel around the caller's element function.
const char *kJitPrologue = R"(
typedef SG_REAL real;
)";

const char *kJitKernel = R"(
struct SgFields { const real *p[8]; };
extern "C" __global__ void __launch_bounds__(128)
sg_jit_rows(int n, const unsigned *__restrict__ ve_ptr, const unsigned *__restrict__ ve_idx,
            const int *__restrict__ ep_all, const unsigned *__restrict__ rowptr,
            const unsigned *__restrict__ colidx, int maxrow, SgFields f,
            real *__restrict__ vals, int *err) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  real *acc_all = reinterpret_cast<real *>(sm);
  real *acc = acc_all + (size_t)warp * maxrow * BS * BS;
  real *stage = acc_all + (size_t)nwarp * maxrow * BS * BS + (size_t)warp * CARD * BS * BS;
  unsigned *cols = reinterpret_cast<unsigned *>(acc_all + (size_t)nwarp * maxrow * BS * BS +
                                                (size_t)nwarp * CARD * BS * BS) +
                   (size_t)warp * maxrow;
  for (long long v = (long long)blockIdx.x * nwarp + warp; v < n;
       v += (long long)gridDim.x * nwarp) {
    const unsigned r0 = rowptr[v], rlen = rowptr[v + 1] - r0;
    if ((int)rlen > maxrow) {
      if (lane == 0) atomicCAS(err, 0, 4);
      continue;
    }
    for (unsigned q = lane; q < rlen; q += 32) cols[q] = colidx[r0 + q];
    for (unsigned q = lane; q < rlen * BS * BS; q += 32) acc[q] = real(0);
    __syncwarp();
    for (unsigned it = ve_ptr[v]; it < ve_ptr[v + 1]; ++it) {
      const unsigned t = ve_idx[it];
      const long long e = t / CARD;
      const int i = (int)(t - (unsigned)e * CARD);
      const int *ep = ep_all + e * CARD;
      int nz = 0;
      if (lane < CARD) {
        real blk[BS][BS];
        for (int a = 0; a < BS; ++a)
          for (int b = 0; b < BS; ++b) blk[a][b] = real(0);
        nz = element_block(e, i, lane, ep, f.p, blk);
        for (int a = 0; a < BS; ++a)
          for (int b = 0; b < BS; ++b) stage[(lane * BS + a) * BS + b] = blk[a][b];
      }
      const unsigned nzmask = __ballot_sync(0xffffffffu, nz != 0);
      __syncwarp();
      if (lane < BS * BS) {
        for (int j = 0; j < CARD; ++j) {
          if (!((nzmask >> j) & 1u)) continue;
          const unsigned col = (unsigned)ep[j];
          unsigned lo = 0, hi = rlen;
          while (lo < hi) {
            const unsigned mid = (lo + hi) >> 1;
            if (cols[mid] < col) lo = mid + 1;
            else hi = mid;
          }
          if (lo >= rlen || cols[lo] != col) {
            atomicCAS(err, 0, 3);
            continue;
          }
          acc[lo * BS * BS + lane] += stage[j * BS * BS + lane];
        }
      }
      __syncwarp();
    }
    for (unsigned q = lane; q < rlen * BS * BS; q += 32) vals[(size_t)r0 * BS * BS + q] = acc[q];
    __syncwarp();
  }
}
)";

struct JitAssembly {
  Ctx *c = nullptr;
  int card = 0, bs = 0, dtype = 0;
  cudaLibrary_t lib = nullptr;
  cudaKernel_t kernel = nullptr;
};

struct JitFields {
  const void *p[JIT_MAX_FIELDS];
};

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" {

int sg_jit_assembly_create(sg_ctx *h, const char *element_src, int32_t card, int32_t bs,
                           int dtype, int32_t exact, sg_jit_assembly **out) {
  Ctx *c = as_ctx(h);
  SG_REQUIRE(c && element_src && out, "sg_jit_assembly_create: null argument");
  SG_REQUIRE(card >= 1 && card <= 32 && bs >= 1 && bs <= 5,
             "sg_jit_assembly_create: card %d bs %d (card 1..32, bs 1..5)", card, bs);
  SG_REQUIRE(dtype == SG_F32 || dtype == SG_F64, "sg_jit_assembly_create: dtype %d", dtype);
  Nvrtc &N = nvrtc();
  if (!N.ok) return set_error(SG_ERR_UNSUPPORTED, "sg_jit_assembly_create: NVRTC not found");
  std::string src = "#define SG_REAL " + std::string(dtype == SG_F64 ? "double" : "float") +
                    "\n#define BS " + std::to_string(bs) + "\n#define CARD " +
                    std::to_string(card) + "\n" + kJitPrologue + "\n" + element_src + "\n" +
                    kJitKernel;
  nvrtcProgram prog = nullptr;
  if (N.create(&prog, src.c_str(), "sg_jit_element.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
    return set_error(SG_ERR_UNSUPPORTED, "sg_jit_assembly_create: nvrtcCreateProgram failed");
  std::vector<const char *> opts = {"-arch=sm_103a", "-std=c++17",
                                    exact ? "--fmad=false" : "--fmad=true"};
  const nvrtcResult rc = N.compile(prog, (int)opts.size(), opts.data());
  if (rc != NVRTC_SUCCESS) {
    size_t ls = 0;
    N.log_size(prog, &ls);
    std::string log(ls, '\0');
    if (ls) N.log(prog, &log[0]);
    N.destroy(&prog);
    if (log.size() > 1500) log.resize(1500);
    return set_error(SG_ERR_ARG, "sg_jit_assembly_create: the element source does not compile:\n%s",
                     log.c_str());
  }
  size_t cs = 0;
  N.cubin_size(prog, &cs);
  std::vector<char> image(cs);
  N.cubin(prog, image.data());
  N.destroy(&prog);
  auto *J = new JitAssembly();
  J->c = c;
  J->card = card;
  J->bs = bs;
  J->dtype = dtype;
  cudaError_t e = cudaLibraryLoadData(&J->lib, image.data(), nullptr, nullptr, 0, nullptr,
                                      nullptr, 0);
  if (e == cudaSuccess) e = cudaLibraryGetKernel(&J->kernel, J->lib, "sg_jit_rows");
  if (e != cudaSuccess) {
    if (J->lib) cudaLibraryUnload(J->lib);
    delete J;
    return set_error(SG_ERR_CUDA, "sg_jit_assembly_create: %s", cudaGetErrorString(e));
  }
  ctx_retain(c);
  *out = reinterpret_cast<sg_jit_assembly *>(J);
  return SG_OK;
}

int sg_jit_assemble(sg_jit_assembly *hj, const sg_mesh *m, const void *const *h_fields,
                    int32_t nfields, void *vals) {
  JitAssembly *J = reinterpret_cast<JitAssembly *>(hj);
  SG_REQUIRE(J && m && vals, "sg_jit_assemble: null argument");
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
  const size_t bb = (size_t)J->bs * J->bs;
  const size_t sh = (size_t)JIT_WARPS * (maxrow * bb * rs + J->card * bb * rs + maxrow * 4);
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
  const int grid = grid_for(c, (int64_t)m->n * 32, JIT_WARPS * 32, 8);
  SG_CHECK_CUDA(cudaLaunchKernel((const void *)J->kernel, dim3(grid), dim3(JIT_WARPS * 32), args,
                                 sh, c->stream));
  return SG_OK;
}

int sg_jit_assembly_destroy(sg_jit_assembly *hj) {
  JitAssembly *J = reinterpret_cast<JitAssembly *>(hj);
  if (!J) return SG_OK;
  cudaStreamSynchronize(J->c->stream);
  if (J->lib) cudaLibraryUnload(J->lib);
  Ctx *c = J->c;
  delete J;
  ctx_release(c);
  return SG_OK;
}

}  // extern "C"
