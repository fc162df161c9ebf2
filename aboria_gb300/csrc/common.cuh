// Shared internals of the aboria_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "abx.h"

namespace abx {

// ---------------------------------------------------------------- errors ---
void set_error(const char *fmt, ...);
void clear_error();

struct Status {
  int code;
};

#define ABX_CHECK_CUDA(expr)                                                  \
  do {                                                                        \
    cudaError_t e__ = (expr);                                                 \
    if (e__ != cudaSuccess) {                                                 \
      ::abx::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,            \
                       cudaGetErrorString(e__));                              \
      return ABX_ERR_CUDA;                                                    \
    }                                                                         \
  } while (0)

#define ABX_REQUIRE(cond, code, ...)                                          \
  do {                                                                        \
    if (!(cond)) {                                                            \
      ::abx::set_error(__VA_ARGS__);                                          \
      return (code);                                                          \
    }                                                                         \
  } while (0)

#define ABX_TRY(...)                                                          \
  do {                                                                        \
    int s__ = (__VA_ARGS__);                                                  \
    if (s__ != ABX_OK) return s__;                                            \
  } while (0)

// ------------------------------------------------------- device buffers ---
// Grow-only device allocation owned by a handle.
template <class T> struct DevBuf {
  T *ptr = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  int reserve(size_t n) {
    if (n <= cap) return ABX_OK;
    release();
    size_t bytes = (n ? n : 1) * sizeof(T);
    cudaError_t e = cudaMalloc((void **)&ptr, bytes);
    if (e != cudaSuccess) {
      ptr = nullptr;
      set_error("cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
      return ABX_ERR_ALLOC;
    }
    cap = n;
    return ABX_OK;
  }
  T *get() const { return ptr; }
};

// Untyped grow-only scratch arena (one per context), carved per call.
struct Scratch {
  DevBuf<unsigned char> buf;
  size_t used = 0;
  // All carving happens on the host before launches; callers reset() at the
  // start of each top-level call.  Sizes are rounded to 256 B.
  void reset() { used = 0; }
};

// ------------------------------------------------------------ context ---
}  // namespace abx

struct abx_context {
  std::atomic<int> refs{1};  // the caller's handle + every object created on it
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
  abx::DevBuf<unsigned char> scratch;   // per-call temporaries
  abx::DevBuf<unsigned char> staging;   // host<->device staging for host pointers
  abx::DevBuf<int> dev_flag;            // device-side error flags
};

namespace abx {

// Carve n elements of T from ctx->scratch at byte offset *off (256 B aligned).
// The caller reserves the total first with scratch_reserve.
template <class T> T *carve(unsigned char *base, size_t &off, size_t n) {
  off = (off + 255) & ~size_t(255);
  T *p = reinterpret_cast<T *>(base + off);
  off += n * sizeof(T);
  return p;
}
template <class T> size_t carve_size(size_t &off, size_t n) {
  off = (off + 255) & ~size_t(255);
  off += n * sizeof(T);
  return off;
}

int ctx_activate(abx_context *ctx);
// Handles are reference counted so that they can be destroyed in any order:
// a context lives while any object created on it does, a particle set while
// any operator built on it does.
void ctx_retain(abx_context *ctx);
void ctx_release(abx_context *ctx);
// Returns 1 if p is device-accessible memory (device or managed), 0 if it is
// host memory (pageable or pinned).
int is_device_ptr(const void *p);
// 1 if p is memory that kernels on `device` may use directly (device memory
// of that GPU, or managed memory), 0 if it is host memory, -1 if it is
// device memory of another GPU.
int device_ptr_usable(const void *p, int device);

// A vector argument that may live on the host or the device.  For host
// pointers a device copy is made (in) or written back (out) around the call.
struct VecArg {
  const void *user = nullptr;
  void *dev = nullptr;
  size_t bytes = 0;
  bool host = false;
};

// ------------------------------------------------------------ kernels ---
inline unsigned int ceil_div(size_t a, size_t b) { return (unsigned int)((a + b - 1) / b); }

// Primitives (primitives.cu)
// Exclusive scan of n uint32 values in place; temp must hold scan_temp_elems(n).
size_t scan_temp_elems(size_t n);
int exclusive_scan_u32(uint32_t *data, size_t n, uint32_t *temp, cudaStream_t s);
// Stable LSD radix sort of (keys, vals) on the low `bits` bits of keys.
// Temp requirements from radix_temp_elems; results end in keys/vals.
size_t radix_temp_u32(size_t n);
int radix_sort_pairs(uint32_t *keys, uint32_t *vals, size_t n, int bits,
                     uint32_t *keys_alt, uint32_t *vals_alt, uint32_t *temp,
                     cudaStream_t s);

}  // namespace abx
