// Dot product that allocates nothing: sg_dot_noalloc.
//
// Who needs this: callers that are not allowed to allocate device memory
// while they run -- a host application that owns and budgets every byte of
// GPU memory itself (a fixed pool handed out by its own allocator), or a
// time-critical loop that must not call cudaMalloc/cudaFree because those
// calls can synchronise the whole device.  Such a caller cannot create an
// sg_ctx (its set-up allocates) and cannot use sg_dot (it takes its partial
// sums from the context's scratch arena, which grows with cudaMalloc).
//
// This entry point keeps its scratch -- one FP64 partial sum per chunk of
// SG_DOT_NOALLOC_CHUNK elements -- in the file-scope device array below,
// whose size is fixed at compile time.  Every GPU that loads the library
// holds the array (512 KB) until the process exits.  Host code cannot use the
// array's name as a device address (in host code it names a host-side
// shadow), so the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current and caches it, and loads
// this file's kernels (with lazy module loading the runtime would otherwise
// load each on its first launch, which can allocate); make that first call
// outside any stream capture and before the stretch that must not allocate.
// `stream` must belong to the device that is current.  All calls share the
// one array: two calls whose kernels overlap on the GPU (different streams,
// no ordering between them) race on it, so order such calls on one stream.
// Each call
// overwrites every partial it later reads, so nothing is carried over from
// the previous call's contents.
#include <mutex>

#include "sg_internal.cuh"

namespace sg {
namespace {

constexpr int NA_THREADS = 256;
constexpr int64_t NA_CHUNK = SG_DOT_NOALLOC_CHUNK;
constexpr int NA_MAX_PARTS = SG_DOT_NOALLOC_MAX_PARTS;

static __device__ __align__(256) double g_dot_parts[NA_MAX_PARTS];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mu;
double *g_na_ptr[NA_MAX_DEVICES] = {};

// Block p sums elements [p*CHUNK, (p+1)*CHUNK) in a fixed order.
template <typename T>
__global__ void __launch_bounds__(NA_THREADS)
    k_dot_chunks(int64_t len, const T *__restrict__ a, const T *__restrict__ b,
                 double *__restrict__ part) {
  __shared__ double sh[NA_THREADS / 32];
  const int64_t base = (int64_t)blockIdx.x * NA_CHUNK;
  int64_t end = base + NA_CHUNK;
  if (end > len) end = len;
  double acc = 0;
  for (int64_t i = base + threadIdx.x; i < end; i += NA_THREADS)
    acc += (double)a[i] * (double)b[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < NA_THREADS / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

// One block: out = sum of the np partials, in a fixed order.
__global__ void __launch_bounds__(NA_THREADS)
    k_dot_final(const double *__restrict__ part, int np, double *__restrict__ out) {
  __shared__ double sh[NA_THREADS / 32];
  double acc = 0;
  for (int i = threadIdx.x; i < np; i += NA_THREADS) acc += part[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < NA_THREADS / 32) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *out = v;
  }
}

// Device address of g_dot_parts on the current device (looked up once).
int scratch_ptr(double **out) {
  int dev = 0;
  SG_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NA_MAX_DEVICES)
    return set_error(SG_ERR_UNSUPPORTED, "sg_dot_noalloc: device %d beyond %d", dev,
                     NA_MAX_DEVICES);
  std::lock_guard<std::mutex> lock(g_na_mu);
  if (!g_na_ptr[dev]) {
    double *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_dot_parts);
    if (e != cudaSuccess || !p)
      return set_error(SG_ERR_CUDA, "sg_dot_noalloc: cudaGetSymbolAddress failed: %s",
                       cudaGetErrorString(e));
    // load the kernels now rather than at their first launch
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, k_dot_chunks<float>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_dot_chunks<double>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_dot_final);
    if (e != cudaSuccess)
      return set_error(SG_ERR_CUDA, "sg_dot_noalloc: loading the kernels failed: %s",
                       cudaGetErrorString(e));
    g_na_ptr[dev] = p;
  }
  *out = g_na_ptr[dev];
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_dot_noalloc(void *stream, int64_t len, int vec_dtype, const void *a,
                              const void *b, double *d_out) {
  SG_REQUIRE(d_out && (len == 0 || (a && b)), "sg_dot_noalloc: null argument");
  SG_REQUIRE(vec_dtype == SG_F32 || vec_dtype == SG_F64, "sg_dot_noalloc: dtype %d",
             vec_dtype);
  SG_REQUIRE(len >= 0 && len <= SG_DOT_NOALLOC_MAX_LEN,
             "sg_dot_noalloc: len %lld outside [0, %lld] (the static scratch holds %d partial "
             "sums of %lld elements each)",
             (long long)len, (long long)SG_DOT_NOALLOC_MAX_LEN, NA_MAX_PARTS,
             (long long)NA_CHUNK);
  double *parts = nullptr;
  SG_TRY(scratch_ptr(&parts));
  cudaStream_t st = (cudaStream_t)stream;
  const int np = (int)((len + NA_CHUNK - 1) / NA_CHUNK);
  if (np > 0) {
    if (vec_dtype == SG_F64)
      k_dot_chunks<double><<<np, NA_THREADS, 0, st>>>(len, (const double *)a, (const double *)b,
                                                      parts);
    else
      k_dot_chunks<float><<<np, NA_THREADS, 0, st>>>(len, (const float *)a, (const float *)b,
                                                     parts);
    SG_CHECK_LAUNCH();
  }
  k_dot_final<<<1, NA_THREADS, 0, st>>>(parts, np, d_out);
  SG_CHECK_LAUNCH();
  return SG_OK;
}
