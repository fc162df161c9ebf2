// Library-level C ABI: error reporting, version, execution contexts, and the
// host/device staging helpers shared by the other translation units.
#include <cstdarg>

#include "common.cuh"
#include "handles.cuh"

namespace abx {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

void ctx_retain(abx_context *ctx) { ctx->refs.fetch_add(1); }

void ctx_release(abx_context *ctx) {
  if (!ctx || ctx->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->scratch.release();
  ctx->staging.release();
  ctx->dev_flag.release();
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

int ctx_activate(abx_context *ctx) {
  ABX_REQUIRE(ctx, ABX_ERR_INVALID, "null context");
  ABX_CHECK_CUDA(cudaSetDevice(ctx->device));
  return ABX_OK;
}

int is_device_ptr(const void *p) {
  if (!p) return 0;
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear: unregistered host memory on old drivers
    return 0;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

int device_ptr_usable(const void *p, int device) {
  if (!p) return 0;
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (attr.type == cudaMemoryTypeManaged) return 1;
  if (attr.type == cudaMemoryTypeDevice) return attr.device == device ? 1 : -1;
  return 0;
}

int HostStage::in(abx_context *ctx, const void *user, size_t bytes, const void **dev) {
  const int kind = (user && bytes) ? device_ptr_usable(user, ctx->device) : 1;
  ABX_REQUIRE(kind >= 0, ABX_ERR_INVALID,
              "a vector argument is device memory of another GPU than the context's (%d)",
              ctx->device);
  if (kind == 1) {
    *dev = user;
    return ABX_OK;
  }
  ABX_TRY(buf.reserve(bytes));
  ABX_CHECK_CUDA(cudaMemcpyAsync(buf.ptr, user, bytes, cudaMemcpyHostToDevice, ctx->stream));
  *dev = buf.ptr;
  return ABX_OK;
}

int HostStage::out(abx_context *ctx, void *user, size_t bytes, void **dev) {
  host_ = false;
  const int kind = (user && bytes) ? device_ptr_usable(user, ctx->device) : 1;
  ABX_REQUIRE(kind >= 0, ABX_ERR_INVALID,
              "a vector argument is device memory of another GPU than the context's (%d)",
              ctx->device);
  if (kind == 1) {
    *dev = user;
    return ABX_OK;
  }
  ABX_TRY(buf.reserve(bytes));
  host_ = true;
  *dev = buf.ptr;
  return ABX_OK;
}

int HostStage::finish(abx_context *ctx, void *user, size_t bytes) {
  if (host_ && bytes) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(user, buf.ptr, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    ABX_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  host_ = false;
  return ABX_OK;
}

}  // namespace abx

using namespace abx;

extern "C" {

const char *abx_last_error(void) { return g_err; }

int abx_version(void) { return 1; }

int abx_context_create(int device, void *stream, abx_context **out) {
  ABX_REQUIRE(out, ABX_ERR_INVALID, "abx_context_create: out is null");
  int ndev = 0;
  ABX_CHECK_CUDA(cudaGetDeviceCount(&ndev));
  ABX_REQUIRE(device >= 0 && device < ndev, ABX_ERR_INVALID,
              "abx_context_create: device %d out of range (%d devices)", device, ndev);
  ABX_CHECK_CUDA(cudaSetDevice(device));
  abx_context *ctx = new abx_context();
  ctx->device = device;
  if (stream) {
    ctx->stream = (cudaStream_t)stream;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete ctx;
      set_error("cudaStreamCreate: %s", cudaGetErrorString(e));
      return ABX_ERR_CUDA;
    }
    ctx->own_stream = true;
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  int st = ctx->dev_flag.reserve(16);
  if (st != ABX_OK) {
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return st;
  }
  cudaMemsetAsync(ctx->dev_flag.ptr, 0, 16 * sizeof(int), ctx->stream);
  *out = ctx;
  clear_error();
  return ABX_OK;
}

int abx_context_destroy(abx_context *ctx) {
  ctx_release(ctx);  // freed once every object created on it is gone
  return ABX_OK;
}

int abx_context_synchronize(abx_context *ctx) {
  ABX_TRY(ctx_activate(ctx));
  ABX_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  return ABX_OK;
}

}  // extern "C"
