// FP32 throughput probe: the denominator of the pair kernels' compute
// roofline, measured on the GPU the library runs on (no counterpart in the
// reference).  A grid of 8 CTAs x 256 threads per SM runs independent FMA
// chains -- 8 per thread, scalar (FFMA) or packed FP32x2 (FFMA2, the form the
// pair kernels use) -- so the FP32 pipe, not latency, limits it; the result is
// timed with CUDA events on the context's stream.
#include "common.cuh"
#include "handles.cuh"

namespace abx {
namespace {

constexpr int PROBE_CHAINS = 8;
constexpr int PROBE_TPB = 256;

template <bool PACKED>
__global__ void __launch_bounds__(PROBE_TPB) k_fp32_probe(float *out, int iters, float m, float c) {
  const float s = 1.0f + 1e-7f * (float)threadIdx.x;
  if (PACKED) {
    float2 v[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) v[k] = make_float2(s + k, s - k);
    const float2 mm = make_float2(m, m), cc = make_float2(c, c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < PROBE_CHAINS; ++k) v[k] = __ffma2_rn(v[k], mm, cc);
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) acc += v[k].x + v[k].y;
    if (acc == 12345.678f) out[blockIdx.x] = acc;  // keeps the chains live
  } else {
    float v[PROBE_CHAINS];
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) v[k] = s + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < PROBE_CHAINS; ++k) v[k] = fmaf(v[k], m, c);
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) acc += v[k];
    if (acc == 12345.678f) out[blockIdx.x] = acc;
  }
}

}  // namespace
}  // namespace abx

using namespace abx;

extern "C" int abx_probe_fp32_peak(abx_context *ctx, int packed, int iters, double *tflops) {
  ABX_REQUIRE(ctx && tflops && iters > 0, ABX_ERR_INVALID, "invalid argument");
  ABX_TRY(ctx_activate(ctx));
  const int blocks = ctx->num_sms * 8;
  DevBuf<float> out;
  ABX_TRY(out.reserve(blocks));
  cudaEvent_t e0, e1;
  ABX_CHECK_CUDA(cudaEventCreate(&e0));
  ABX_CHECK_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int st = ABX_OK;
  for (int rep = 0; rep < 4 && st == ABX_OK; ++rep) {
    cudaEventRecord(e0, ctx->stream);
    if (packed)
      k_fp32_probe<true><<<blocks, PROBE_TPB, 0, ctx->stream>>>(out.ptr, iters, 0.9999f, 1e-4f);
    else
      k_fp32_probe<false><<<blocks, PROBE_TPB, 0, ctx->stream>>>(out.ptr, iters, 0.9999f, 1e-4f);
    cudaEventRecord(e1, ctx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error("fp32 probe: %s", cudaGetErrorString(e));
      st = ABX_ERR_CUDA;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0) best = ms < best ? ms : best;  // first launch is the warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != ABX_OK) return st;
  const double fma_per_chain = packed ? 2.0 : 1.0;
  const double flop = 2.0 * fma_per_chain * PROBE_CHAINS * (double)iters * PROBE_TPB * blocks;
  *tflops = flop / (best * 1e-3) / 1e12;
  return ABX_OK;
}
