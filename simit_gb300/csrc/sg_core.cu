// Context, errors, scratch arena, scan and dot.
#include <stdlib.h>
#include <string.h>

#include "sg_internal.cuh"

namespace sg {

static thread_local std::string g_last_error;

int set_error(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int Scratch::reserve(size_t bytes) {
  bytes = (bytes + 255) & ~size_t(255);
  if (bytes <= c_->arena_bytes) return SG_OK;
  SG_CHECK_CUDA(cudaStreamSynchronize(c_->stream));
  if (c_->arena) SG_CHECK_CUDA(cudaFree(c_->arena));
  c_->arena = nullptr;
  c_->arena_bytes = 0;
  size_t grow = bytes + bytes / 4;
  SG_CHECK_CUDA(cudaMalloc(&c_->arena, grow));
  c_->arena_bytes = grow;
  return SG_OK;
}

int check_device_error(Ctx *c, const char *what) {
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int),
                                cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  int e = *c->h_err;
  if (e != DEV_OK) {
    SG_CHECK_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
    static const char *names[] = {"ok", "endpoint outside [0, n)",
                                  "row candidate list exceeds sort capacity",
                                  "(row, col) not in pattern",
                                  "row longer than the assembly accumulator",
                                  "vertex without a diagonal block",
                                  "bulk-copy barrier wait timed out",
                                  "an element needs more than 128 colours",
                                  "bulk copies still in flight after a timeout (results "
                                  "undefined; destroy and recreate the context)"};
    const char *nm = (e > 0 && e < 9) ? names[e] : "unknown";
    return set_error(SG_ERR_DEVICE, "%s: device check failed (%d: %s)", what, e,
                     nm);
  }
  return SG_OK;
}

// ---------------------------------------------------------------------------
// Exclusive scan (three phases; block sums scanned recursively).
// ---------------------------------------------------------------------------
constexpr int SCAN_T = 512;       // threads per block
constexpr int SCAN_PER = 8;       // items per thread
constexpr int SCAN_TILE = SCAN_T * SCAN_PER;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the prefix and
// the block total through *total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *total) {
  __shared__ uint32_t wsum[SCAN_T / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = warp_incl_scan(v);
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t s = (lane < SCAN_T / 32) ? wsum[lane] : 0;
    uint32_t si = warp_incl_scan(s);
    if (lane < SCAN_T / 32) wsum[lane] = si - s;
    if (lane == SCAN_T / 32 - 1) *total = si;
  }
  __syncthreads();
  uint32_t r = inc - v + wsum[w];
  __syncthreads();
  return r;
}

__global__ void scan_tile_sums(const uint32_t *in, int64_t n, uint32_t *sums) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  uint32_t acc = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k) {
    int64_t i = base + (int64_t)k * SCAN_T + threadIdx.x;
    if (i < n) acc += in[i];
  }
  __shared__ uint32_t tot;
  block_excl_scan(acc, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// Each thread scans SCAN_PER consecutive items; `offs` (may be null) holds
// the exclusive prefix of each tile.  out has n+1 entries when last_total.
__global__ void scan_tiles(const uint32_t *in, int64_t n, const uint32_t *offs,
                           uint32_t *out, int write_total) {
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_PER;
  uint32_t v[SCAN_PER];
  uint32_t acc = 0;
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k) {
    int64_t i = base + k;
    v[k] = (i < n) ? in[i] : 0;
    acc += v[k];
  }
  __shared__ uint32_t tot;
  uint32_t pre = block_excl_scan(acc, &tot);
  uint32_t off = (offs ? offs[blockIdx.x] : 0) + pre;
#pragma unroll
  for (int k = 0; k < SCAN_PER; ++k) {
    int64_t i = base + k;
    if (i < n) out[i] = off;
    off += v[k];
  }
  if (write_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
    out[n] = (offs ? offs[blockIdx.x] : 0) + tot;
}

size_t scan_scratch_bytes(int64_t n) {
  size_t total = 0;
  while (n > SCAN_TILE) {
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    total += Scratch::bytes_for(tiles + 1, 4) * 2;
    n = tiles;
  }
  return total + 256;
}

int exclusive_scan_u32(Ctx *c, Scratch &s, const uint32_t *in, uint32_t *out,
                       int64_t n) {
  if (n <= 0) {
    SG_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), c->stream));
    return SG_OK;
  }
  int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles == 1) {
    scan_tiles<<<1, SCAN_T, 0, c->stream>>>(in, n, nullptr, out, 1);
    SG_CHECK_LAUNCH();
    return SG_OK;
  }
  uint32_t *sums = s.alloc<uint32_t>(tiles + 1);
  uint32_t *offs = s.alloc<uint32_t>(tiles + 1);
  scan_tile_sums<<<(unsigned)tiles, SCAN_T, 0, c->stream>>>(in, n, sums);
  SG_CHECK_LAUNCH();
  SG_TRY(exclusive_scan_u32(c, s, sums, offs, tiles));
  scan_tiles<<<(unsigned)tiles, SCAN_T, 0, c->stream>>>(in, n, offs, out, 1);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// ---------------------------------------------------------------------------
// Deterministic FP64 dot: fixed grid, per-block partials, one final block.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void dot_partials(int64_t len, const T *a, const T *b, double *part) {
  double acc = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x)
    acc += (double)a[i] * (double)b[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? ws[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
  }
}

__global__ void sum_partials(const double *part, int np, double *out) {
  double acc = 0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) acc += part[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? ws[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *out = v;
  }
}

template <typename T>
__global__ void k_axpy(int64_t len, T alpha, const T *__restrict__ x, T *__restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len;
       i += (int64_t)gridDim.x * blockDim.x) {
    // separate rounding of the product and the sum (no contraction)
    if (sizeof(T) == 8)
      y[i] = (T)__dadd_rn((double)y[i], __dmul_rn((double)alpha, (double)x[i]));
    else
      y[i] = (T)__fadd_rn((float)y[i], __fmul_rn((float)alpha, (float)x[i]));
  }
}

void ctx_release(Ctx *c) {
  if (--c->refs > 0) return;
  cudaStreamSynchronize(c->stream);
  if (c->arena) cudaFree(c->arena);
  if (c->d_err) cudaFree(c->d_err);
  if (c->h_err) cudaFreeHost(c->h_err);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  cudaStreamDestroy(c->stream);
  delete c;
}

// FP64 FMA rate probe: eight independent FMA chains per thread, so the FP64
// pipe, not latency, bounds it.  The sum is stored so that nothing is
// optimised away.
__global__ void k_fma_rate(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace sg

using namespace sg;

extern "C" {

int sg_ctx_create(int device, sg_ctx **out) {
  if (!out) return set_error(SG_ERR_ARG, "sg_ctx_create: out is null");
  int ndev = 0;
  SG_CHECK_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev)
    return set_error(SG_ERR_ARG, "sg_ctx_create: device %d of %d", device, ndev);
  // the context's device is current while it is set up; the caller's
  // current device is restored on return
  DeviceGuardT<CudaDeviceApi> dg_(device);
  Ctx *c = new Ctx();
  c->device = device;
  SG_CHECK_CUDA(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
  SG_CHECK_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  SG_CHECK_CUDA(cudaMalloc(&c->d_err, 64));
  SG_CHECK_CUDA(cudaMemsetAsync(c->d_err, 0, 64, c->stream));
  SG_CHECK_CUDA(cudaMallocHost(&c->h_err, 64));
  SG_CHECK_CUDA(cudaMallocHost(&c->h_stage, 1 << 16));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  *out = reinterpret_cast<sg_ctx *>(c);
  return SG_OK;
}

int sg_ctx_destroy(sg_ctx *h) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  if (!c) return SG_OK;
  ctx_release(c);
  return SG_OK;
}

int sg_ctx_sync(sg_ctx *h) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  if (!c) return set_error(SG_ERR_ARG, "sg_ctx_sync: null context");
  return check_device_error(c, "sg_ctx_sync");
}

void *sg_ctx_stream(sg_ctx *h) { return h ? (void *)as_ctx(h)->stream : nullptr; }

const char *sg_last_error(void) { return g_last_error.c_str(); }

const char *sg_version(void) { return "simit_gb300 0.1 (sm_103a)"; }

int sg_axpy(sg_ctx *h, int64_t len, int vdt, double alpha, const void *x, void *y) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && (len == 0 || (x && y)), "sg_axpy: null argument");
  SG_REQUIRE(len >= 0 && (vdt == SG_F32 || vdt == SG_F64), "sg_axpy: bad len/dtype");
  if (len == 0) return SG_OK;
  const int G = grid_for(c, len, 256, 8);
  if (vdt == SG_F64)
    k_axpy<double><<<G, 256, 0, c->stream>>>(len, alpha, (const double *)x, (double *)y);
  else
    k_axpy<float><<<G, 256, 0, c->stream>>>(len, (float)alpha, (const float *)x, (float *)y);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

int sg_dot(sg_ctx *h, int64_t len, int vdt, const void *a, const void *b,
           double *h_out) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && a && b && h_out, "sg_dot: null argument");
  SG_REQUIRE(len >= 0 && (vdt == SG_F32 || vdt == SG_F64), "sg_dot: bad len/dtype");
  const int T = 256;
  const int G = grid_for(c, len, T, 4);
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for(G, 8) + 256));
  double *part = s.alloc<double>(G);
  double *res = s.alloc<double>(1);
  if (vdt == SG_F64)
    dot_partials<double><<<G, T, 0, c->stream>>>(len, (const double *)a, (const double *)b, part);
  else
    dot_partials<float><<<G, T, 0, c->stream>>>(len, (const float *)a, (const float *)b, part);
  SG_CHECK_LAUNCH();
  sum_partials<<<1, 256, 0, c->stream>>>(part, G, res);
  SG_CHECK_LAUNCH();
  SG_CHECK_CUDA(cudaMemcpyAsync(c->h_stage, res, 8, cudaMemcpyDeviceToHost, c->stream));
  SG_CHECK_CUDA(cudaStreamSynchronize(c->stream));
  *h_out = *(double *)c->h_stage;
  return SG_OK;
}

int sg_fp64_fma_rate(sg_ctx *h, double *tflops) {
  Ctx *c = as_ctx(h);
  DeviceGuard dg_(c);
  SG_REQUIRE(c && tflops, "sg_fp64_fma_rate: null argument");
  const int T = 256, G = c->num_sms * 8, iters = 4096, reps = 5;
  Scratch s(c);
  SG_TRY(s.reserve(Scratch::bytes_for((int64_t)G * T, 8) + 256));
  double *out = s.alloc<double>((int64_t)G * T);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  SG_CHECK_CUDA(cudaEventCreate(&e0));
  cudaError_t e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    k_fma_rate<<<G, T, 0, c->stream>>>(out, iters, 0.999999, 1e-7);  // warm-up
    e = cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r)
      k_fma_rate<<<G, T, 0, c->stream>>>(out, iters, 0.999999, 1e-7);
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  }
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  SG_CHECK_CUDA(e);
  *tflops = 2.0 * 8.0 * iters * (double)G * T * reps / (ms * 1e-3) / 1e12;
  return SG_OK;
}

}  // extern "C"
