// Internal helpers shared by the simit_gb300 CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdarg.h>
#include <stdio.h>

#include <mutex>
#include <string>

#include "../../include/simit_gb300.h"
#include "sg_device_guard.h"

namespace sg {

// Per-context state: the stream every call is ordered on, a grow-only device
// scratch arena, a device error word and pinned host staging.
// Per-device one-time flags (function attributes and occupancy are properties
// of a device's context, not of the process).
constexpr int SG_MAX_DEVICES = 64;
// Runs `init` once per device and returns its status on every call; a
// thread that arrives while another runs it waits for it to finish, so no
// launch can overtake the attribute it depends on.
struct PerDeviceOnce {
  std::once_flag flag[SG_MAX_DEVICES];
  int rc[SG_MAX_DEVICES] = {};
};
template <typename F> inline int once_per_device(PerDeviceOnce &o, int device, F &&init) {
  if (device < 0 || device >= SG_MAX_DEVICES) return init();
  std::call_once(o.flag[device], [&] { o.rc[device] = init(); });
  return o.rc[device];
}

struct Ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  char *arena = nullptr;
  size_t arena_bytes = 0;
  int *d_err = nullptr;      // device error word (0 = ok), see ErrCode below
  int *h_err = nullptr;      // pinned mirror
  void *h_stage = nullptr;   // pinned staging (64 KB)
  // (rowptr, n) -> longest row, for kernels that size shared memory by it
  static constexpr int MAXROW_CACHE = 8;
  const uint32_t *mr_ptr[MAXROW_CACHE] = {};
  int32_t mr_n[MAXROW_CACHE] = {};
  int32_t mr_val[MAXROW_CACHE] = {};
  int32_t mr_t16[MAXROW_CACHE] = {};  // largest 16-row tile, in blocks
  int32_t mr_t32[MAXROW_CACHE] = {};  // largest 32-row tile, in blocks
  int32_t mr_t4[MAXROW_CACHE] = {};   // largest 4-row tile
  int32_t mr_t8[MAXROW_CACHE] = {};   // largest 8-row tile
  int mr_next = 0;
  int refs = 1;  // sg_ctx_destroy + one per live solver
  // Set while a solver captures its iteration graph: kernels launched with
  // launch_k then carry programmatic stream serialisation, so each may start
  // while its predecessor drains (the kernels wait with griddepcontrol.wait
  // before their first global access).
  bool pdl = false;
};

// Kernel launch honouring Ctx::pdl (cudaLaunchKernelEx with the
// programmatic-stream-serialisation attribute when it is set).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(const Ctx *c, void (*kern)(KArgs...), dim3 grid, dim3 block,
                            size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  if (c->pdl) {
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  return cudaLaunchKernelEx(&cfg, kern, args...);
}

// Drops one reference; frees the context when none are left.
void ctx_release(Ctx *c);
inline void ctx_retain(Ctx *c) { ++c->refs; }

// Device-side error codes written to Ctx::d_err by bounds checks.
enum DevErr : int {
  DEV_OK = 0,
  DEV_BAD_ENDPOINT = 1,   // endpoint outside [0, n)
  DEV_ROW_TOO_LONG = 2,   // candidate list exceeds the sort capacity
  DEV_SLOT_MISSING = 3,   // (row, col) not found in the pattern
  DEV_ROW_OVERFLOW = 4,   // assembly row longer than the accumulator
  DEV_NO_DIAGONAL = 5,    // vertex without a diagonal block
  DEV_TMA_TIMEOUT = 6,    // a bulk-copy barrier wait ran out of polls
  DEV_TOO_MANY_COLORS = 7,  // element colouring needs more than SG_MAX_COLORS
  DEV_TMA_UNDRAINED = 8,    // after a timeout, a copy was still in flight at exit:
                            // results undefined, reset the context
};

int set_error(int code, const char *fmt, ...);

#define SG_CHECK_CUDA(call)                                                   \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return ::sg::set_error(SG_ERR_CUDA, "%s failed: %s (%s:%d)", #call,     \
                             cudaGetErrorString(e_), __FILE__, __LINE__);     \
  } while (0)

#define SG_CHECK_LAUNCH() SG_CHECK_CUDA(cudaGetLastError())

#define SG_REQUIRE(cond, ...)                                                 \
  do {                                                                        \
    if (!(cond)) return ::sg::set_error(SG_ERR_ARG, __VA_ARGS__);             \
  } while (0)

#define SG_TRY(expr)                                                          \
  do {                                                                        \
    int rc_ = (expr);                                                         \
    if (rc_ != SG_OK) return rc_;                                             \
  } while (0)

// Bump allocator over the context arena.  reserve() must be called with the
// total size before any alloc() of one call; the arena only grows (with a
// stream sync before the old block is released).
class Scratch {
 public:
  explicit Scratch(Ctx *c) : c_(c) {}
  int reserve(size_t bytes);
  template <typename T> T *alloc(size_t count) {
    size_t off = (used_ + 255) & ~size_t(255);
    used_ = off + count * sizeof(T);
    return reinterpret_cast<T *>(c_->arena + off);
  }
  static size_t bytes_for(size_t count, size_t elem) {
    return ((count * elem) + 255) & ~size_t(255);
  }

 private:
  Ctx *c_;
  size_t used_ = 0;
};

// Reads back and clears the device error word (synchronises the stream).
int check_device_error(Ctx *c, const char *what);

// Exclusive scan of n uint32 counts into out[0..n] (out[n] = total), using
// scratch from `s` (at most scan_scratch_bytes(n)).  Returns the total
// through *total_host when non-null (synchronises).
size_t scan_scratch_bytes(int64_t n);
int exclusive_scan_u32(Ctx *c, Scratch &s, const uint32_t *in, uint32_t *out,
                       int64_t n);

// Number of blocks for a grid-stride kernel: `per_sm` blocks on every SM.
inline int grid_for(const Ctx *c, int64_t work_items, int threads, int per_sm) {
  int64_t need = (work_items + threads - 1) / threads;
  int64_t cap = (int64_t)c->num_sms * per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

inline Ctx *as_ctx(sg_ctx *h) { return reinterpret_cast<Ctx *>(h); }

struct CudaDeviceApi {
  static bool get(int *d) { return cudaGetDevice(d) == cudaSuccess; }
  static bool set(int d) { return cudaSetDevice(d) == cudaSuccess; }
};
// Makes the context's device current for one entry point (see
// sg_device_guard.h); a null context is a no-op.
struct DeviceGuard : DeviceGuardT<CudaDeviceApi> {
  explicit DeviceGuard(const Ctx *c) : DeviceGuardT<CudaDeviceApi>(c ? c->device : -1) {}
};

// dtype helpers
inline size_t dtype_size(int dt) { return dt == SG_F64 ? 8 : 4; }

}  // namespace sg
