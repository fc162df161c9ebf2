// Learned sparse-approximate-inverse model: a small MLP mapping a particle's
// k-nearest-neighbour geometry (relative positions scaled by the kernel's
// shape parameter) to that particle's k approximate-inverse weights.  There is
// no counterpart in the reference; its training labels are the exact
// least-squares rows of CardinalFunctionsPreconditioner::factorize
// (src/Preconditioners.h:1025-1082) on the same support (spai.cu).
//
// Training runs in FP32 with hand-written kernels: a tiled SIMT GEMM with
// transpose flags and fused bias/activation (forward, dX = dZ W^T,
// dW = X^T dZ), column sums for bias gradients, SiLU derivative, MSE loss and
// Adam.  Inference uses BF16 weights/activations on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation) with the whole network evaluated
// per 64-point tile in shared memory.
//
// Parameter layout (flat FP32): for each layer l, W_l [in_l x out_l]
// row-major, then b_l [out_l].  Hidden layers use SiLU, the output is
// linear, followed by y = y * out_scale + out_shift (target normalisation).
#include <cmath>
#include <cstdio>
#include <cuda_bf16.h>
#include <vector>

#include "common.cuh"
#include "handles.cuh"

struct abx_mlp {
  abx_context *ctx = nullptr;
  int nlayers = 0;           // linear layers (hidden + output)
  std::vector<int> dims;     // nlayers + 1
  std::vector<size_t> woff, boff;
  size_t nparams = 0;
  abx::DevBuf<float> params, grads, m1, m2;
  abx::DevBuf<float> out_scale, out_shift;
  float in_scale = 1.0f;
  int out_transform = 0;  // 0: y; 1: out_c * sinh(y) (targets trained as asinh(w / out_c))
  float out_c = 1.0f;
  int loss_kind = ABX_LOSS_MSE;
  int loss_dim = 0;         // ABX_LOSS_SPAI_RESIDUAL: coordinates per support point
  abx_kernel loss_kern{};   //   kernel and cut-off in feature units
  float loss_cut2 = 0.f;
  int64_t step = 0;
  // activations for the last batch (training)
  abx::DevBuf<float> act, pre;  // sum over layers of B*dims
  abx::DevBuf<float> dbuf0, dbuf1, lossbuf;
  int64_t cap_batch = 0;
  // inference weights: BF16, transposed [out][in_pad]
  abx::DevBuf<__nv_bfloat16> wt16;
  std::vector<size_t> wt_off;
  std::vector<int> in_pad;
  bool infer_ready = false;
  abx::HostStage sx, sy;
};

namespace abx {
namespace {

constexpr int GT = 64;  // GEMM tile
constexpr int GK = 16;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// C[M x N] (+)= op(A) op(B) (+ bias), op(A)(m,k) = TA ? A[k*lda + m] : A[m*lda + k],
// op(B)(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n].  Epilogue: ACT 0 none, 1 SiLU
// (pre-activation stored to Z when given).  ACC: C += result.
template <bool TA, bool TB, int ACT, bool ACC>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float *__restrict__ A,
                                              int lda, const float *__restrict__ B, int ldb,
                                              const float *__restrict__ bias,
                                              float *__restrict__ Z, float *__restrict__ C,
                                              int ldc) {
  __shared__ float sA[GK][GT + 1];
  __shared__ float sB[GK][GT + 1];
  const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
  const int tid = threadIdx.x;
  const int tr = (tid / 16) * 4, tc = (tid % 16) * 4;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += GK) {
    for (int e = tid; e < GK * GT; e += 256) {
      const int kk = e / GT, mm = e % GT;
      const int m = m0 + mm, k = k0 + kk;
      sA[kk][mm] = (m < M && k < K) ? (TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k]) : 0.f;
      const int n = n0 + mm;
      sB[kk][mm] = (n < N && k < K) ? (TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n]) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][tr + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][tc + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tr + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tc + j;
      if (n >= N) continue;
      float v = acc[i][j] + (bias ? bias[n] : 0.f);
      if (ACT == 1) {
        if (Z) Z[(size_t)m * ldc + n] = v;
        v = silu(v);
      }
      if (ACC) v += C[(size_t)m * ldc + n];
      C[(size_t)m * ldc + n] = v;
    }
  }
}

template <bool TA, bool TB, int ACT, bool ACC>
void gemm(cudaStream_t s, int M, int N, int K, const float *A, int lda, const float *B, int ldb,
          const float *bias, float *Z, float *C, int ldc) {
  dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT);
  k_gemm<TA, TB, ACT, ACC><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, bias, Z, C, ldc);
}

// dY -> dZ = dY * silu'(Z)
__global__ void k_silu_back(int64_t n, const float *__restrict__ Z, float *__restrict__ d) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] *= silu_grad(Z[i]);
}

// column sums: out[n] = sum_m X[m*N + n]
__global__ void k_colsum(int M, int N, const float *__restrict__ X, float *__restrict__ out) {
  const int n = blockIdx.x;
  float s = 0.f;
  for (int m = threadIdx.x; m < M; m += blockDim.x) s += X[(size_t)m * N + n];
  __shared__ float red[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int i = 0; i < (int)blockDim.x / 32; ++i) t += red[i];
    out[n] = t;
  }
}

// MSE on normalised targets: t_n = (y - shift) / scale; d = 2 (out - t) / (M*N)
__global__ void k_mse(int64_t n, int N, const float *__restrict__ out,
                      const float *__restrict__ target, const float *__restrict__ scale,
                      const float *__restrict__ shift, float *__restrict__ d,
                      float *__restrict__ loss) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.f;
  if (i < n) {
    const int c = (int)(i % N);
    const float t = (target[i] - shift[c]) / scale[c];
    const float e = out[i] - t;
    d[i] = 2.f * e / (float)n;
    l = e * e / (float)n;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.f) atomicAdd(loss, l);
}

__device__ __forceinline__ float kern_feature(const abx_kernel &k, float d2) {
  switch (k.kind) {
  case ABX_K_CONST: return (float)k.p[0];
  case ABX_K_GAUSSIAN:
  case ABX_K_COMPACT_GAUSSIAN: return __expf(-d2 * (float)k.p[0]);
  case ABX_K_WENDLAND_C2: {
    const float q = sqrtf(d2) * (float)k.p[0];
    const float t = fmaxf(1.f - q, 0.f), t2 = t * t;
    return t2 * t2 * (4.f * q + 1.f);
  }
  case ABX_K_LAPLACE: return 1.f / (sqrtf(d2) + (float)k.p[0]);
  case ABX_K_MULTIQUADRIC: return sqrtf(d2 + (float)k.p[0]);
  default: return 0.f;
  }
}

// Approximate-inverse residual loss, one warp per row (k <= 32 support
// points, lane a holds point a): m = out * scale + shift, r = A m - e_0,
// loss += |r|^2 / B, d = scale * 2 A r / B (A symmetric).
__global__ void k_spai_residual(int64_t B, int k, int dim, abx_kernel kern, float cut2,
                                const float *__restrict__ feats, const float *__restrict__ out,
                                const float *__restrict__ scale, const float *__restrict__ shift,
                                float *__restrict__ d, float *__restrict__ loss) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int a = threadIdx.x & 31;
  if (row >= B) return;  // whole warps exit together
  const bool act = a < k;
  float f[3] = {0.f, 0.f, 0.f};
  for (int e = 0; e < dim; ++e) f[e] = act ? feats[(row * k + a) * dim + e] : 0.f;
  const float m = act ? out[row * k + a] * scale[a] + shift[a] : 0.f;
  float am = 0.f;
  for (int b = 0; b < k; ++b) {
    float d2 = 0.f;
    for (int e = 0; e < dim; ++e) {
      const float v = __shfl_sync(0xffffffffu, f[e], b) - f[e];
      d2 = fmaf(v, v, d2);
    }
    const float mb = __shfl_sync(0xffffffffu, m, b);
    const float A = (cut2 <= 0.f || d2 < cut2) ? kern_feature(kern, d2) : 0.f;
    am = fmaf(A, mb, am);
  }
  const float r = act ? am - (a == 0 ? 1.f : 0.f) : 0.f;
  float ar = 0.f;
  for (int b = 0; b < k; ++b) {
    float d2 = 0.f;
    for (int e = 0; e < dim; ++e) {
      const float v = __shfl_sync(0xffffffffu, f[e], b) - f[e];
      d2 = fmaf(v, v, d2);
    }
    const float rb = __shfl_sync(0xffffffffu, r, b);
    const float A = (cut2 <= 0.f || d2 < cut2) ? kern_feature(kern, d2) : 0.f;
    ar = fmaf(A, rb, ar);
  }
  if (act) d[row * k + a] = scale[a] * 2.f * ar / (float)B;
  float l = r * r / (float)B;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if (a == 0) atomicAdd(loss, l);
}

__global__ void k_adam(int64_t n, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_scale_in(int64_t n, const float *__restrict__ x, float s, float *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] * s;
}

__global__ void k_denorm(int64_t n, int N, float *__restrict__ y, const float *__restrict__ scale,
                         const float *__restrict__ shift, int transform, float oc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const int c = (int)(i % N);
    const float v = y[i] * scale[c] + shift[c];
    y[i] = transform ? oc * sinhf(v) : v;
  }
}

// ---------------------------------------------------- BF16 tensor cores ---
constexpr int IT = 64;      // points per CTA
constexpr int IW = 4;       // warps per CTA (16 rows each)
constexpr int IMAXW = 128;  // max layer width handled

__global__ void k_transpose_bf16(const float *__restrict__ W, int in, int out, int in_pad,
                                 __nv_bfloat16 *__restrict__ Wt) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= out * in_pad) return;
  const int o = idx / in_pad, i = idx % in_pad;
  Wt[idx] = __float2bfloat16(i < in ? W[(size_t)i * out + o] : 0.f);
}

struct InferParams {
  int nlayers;
  int dims[8];
  int in_pad[8];
  const __nv_bfloat16 *wt[8];
  const float *bias[8];
  const float *x;
  float in_scale;
  int64_t n;
  float *y;
  const float *out_scale, *out_shift;
  int out_transform;
  float out_c;
};

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Whole-network inference for 64 points per CTA.  Activations ping-pong
// between two shared BF16 buffers [64][IMAXW+8]; each warp owns 16 rows and
// produces all output columns of a layer with m16n8k16 MMAs reading the
// layer's transposed BF16 weights from global memory (L1/L2 resident).
__global__ void __launch_bounds__(IW * 32) k_mlp_infer_bf16(InferParams P) {
  constexpr int LD = IMAXW + 8;  // padded row (bf16 elements)
  __shared__ __align__(16) __nv_bfloat16 buf[2][IT][LD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int64_t p0 = (int64_t)blockIdx.x * IT;
  // input tile (scaled), zero padded to in_pad[0]
  const int in0 = P.dims[0], ip0 = P.in_pad[0];
  for (int e = tid; e < IT * ip0; e += IW * 32) {
    const int r = e / ip0, c = e % ip0;
    const int64_t pt = p0 + r;
    const float v = (pt < P.n && c < in0) ? P.x[pt * in0 + c] * P.in_scale : 0.f;
    buf[0][r][c] = __float2bfloat16(v);
  }
  __syncthreads();
  int cur = 0;
  const int row0 = warp * 16;
  for (int l = 0; l < P.nlayers; ++l) {
    const int K = P.in_pad[l], N = P.dims[l + 1];
    const __nv_bfloat16 *Wt = P.wt[l];
    const bool last = l == P.nlayers - 1;
    const int npad_next = last ? 0 : P.in_pad[l + 1];
    for (int n0 = 0; n0 < N; n0 += 8) {
      float c[4] = {0.f, 0.f, 0.f, 0.f};
      for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4], b[2];
        a[0] = *(const uint32_t *)&buf[cur][row0 + g][k0 + 2 * t];
        a[1] = *(const uint32_t *)&buf[cur][row0 + g + 8][k0 + 2 * t];
        a[2] = *(const uint32_t *)&buf[cur][row0 + g][k0 + 2 * t + 8];
        a[3] = *(const uint32_t *)&buf[cur][row0 + g + 8][k0 + 2 * t + 8];
        const __nv_bfloat16 *wr = Wt + (size_t)(n0 + g) * K + k0 + 2 * t;
        b[0] = *(const uint32_t *)wr;
        b[1] = *(const uint32_t *)(wr + 8);
        mma_bf16(c, a, b);
      }
      const int col = n0 + 2 * t;
      const float b0 = P.bias[l][col], b1 = P.bias[l][col + 1];
      float v[4] = {c[0] + b0, c[1] + b1, c[2] + b0, c[3] + b1};
      if (!last) {
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = silu(v[q]);
        buf[cur ^ 1][row0 + g][col] = __float2bfloat16(v[0]);
        buf[cur ^ 1][row0 + g][col + 1] = __float2bfloat16(v[1]);
        buf[cur ^ 1][row0 + g + 8][col] = __float2bfloat16(v[2]);
        buf[cur ^ 1][row0 + g + 8][col + 1] = __float2bfloat16(v[3]);
      } else {
        const int64_t ra = p0 + row0 + g, rb = ra + 8;
        const float s0 = P.out_scale[col], s1 = P.out_scale[col + 1];
        const float h0 = P.out_shift[col], h1 = P.out_shift[col + 1];
        float o[4] = {v[0] * s0 + h0, v[1] * s1 + h1, v[2] * s0 + h0, v[3] * s1 + h1};
        if (P.out_transform)
#pragma unroll
          for (int q = 0; q < 4; ++q) o[q] = P.out_c * sinhf(o[q]);
        if (ra < P.n) {
          P.y[ra * N + col] = o[0];
          P.y[ra * N + col + 1] = o[1];
        }
        if (rb < P.n) {
          P.y[rb * N + col] = o[2];
          P.y[rb * N + col + 1] = o[3];
        }
      }
    }
    if (!last) {
      // zero the padding columns of the next layer's input
      for (int e = tid; e < IT * (npad_next - N); e += IW * 32) {
        const int r = e / (npad_next - N), cc = N + e % (npad_next - N);
        buf[cur ^ 1][r][cc] = __float2bfloat16(0.f);
      }
    }
    __syncthreads();
    cur ^= 1;
  }
}

__global__ void k_init_uniform(float *p, int64_t n, float a, uint64_t seed) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const float u = (float)((z >> 40) * (1.0 / 16777216.0));
  p[i] = (2.f * u - 1.f) * a;
}

int mlp_reserve_batch(abx_mlp *M, int64_t B) {
  if (B <= M->cap_batch) return ABX_OK;
  size_t tot = 0;
  for (int d : M->dims) tot += (size_t)B * d;
  ABX_TRY(M->act.reserve(tot));
  ABX_TRY(M->pre.reserve(tot));
  int mx = 0;
  for (int d : M->dims) mx = std::max(mx, d);
  ABX_TRY(M->dbuf0.reserve((size_t)B * mx));
  ABX_TRY(M->dbuf1.reserve((size_t)B * mx));
  ABX_TRY(M->lossbuf.reserve(4));
  M->cap_batch = B;
  return ABX_OK;
}

// forward in FP32 keeping activations (act[l] = input of layer l, pre[l+1]).
int mlp_forward32(abx_mlp *M, const float *x, int64_t B) {
  cudaStream_t s = M->ctx->stream;
  ABX_TRY(mlp_reserve_batch(M, B));
  std::vector<size_t> aoff(M->nlayers + 1);
  size_t o = 0;
  for (int l = 0; l <= M->nlayers; ++l) {
    aoff[l] = o;
    o += (size_t)B * M->dims[l];
  }
  float *act = M->act.ptr, *pre = M->pre.ptr;
  k_scale_in<<<ceil_div((size_t)B * M->dims[0], 256), 256, 0, s>>>((size_t)B * M->dims[0], x,
                                                                   M->in_scale, act);
  for (int l = 0; l < M->nlayers; ++l) {
    const int in = M->dims[l], out = M->dims[l + 1];
    const float *W = M->params.ptr + M->woff[l];
    const float *b = M->params.ptr + M->boff[l];
    if (l < M->nlayers - 1)
      gemm<false, false, 1, false>(s, (int)B, out, in, act + aoff[l], in, W, out, b,
                                   pre + aoff[l + 1], act + aoff[l + 1], out);
    else
      gemm<false, false, 0, false>(s, (int)B, out, in, act + aoff[l], in, W, out, b, nullptr,
                                   act + aoff[l + 1], out);
  }
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

// gradients of the normalised-target MSE into M->grads; returns the loss.
int mlp_backward(abx_mlp *M, const float *x, const float *target, int64_t B, float *loss) {
  cudaStream_t s = M->ctx->stream;
  ABX_TRY(mlp_forward32(M, x, B));
  std::vector<size_t> aoff(M->nlayers + 1);
  size_t o = 0;
  for (int l = 0; l <= M->nlayers; ++l) {
    aoff[l] = o;
    o += (size_t)B * M->dims[l];
  }
  const int L = M->nlayers;
  const int nout = M->dims[L];
  float *d = M->dbuf0.ptr, *dn = M->dbuf1.ptr;
  ABX_CHECK_CUDA(cudaMemsetAsync(M->lossbuf.ptr, 0, sizeof(float), s));
  if (M->loss_kind == ABX_LOSS_SPAI_RESIDUAL)
    k_spai_residual<<<ceil_div((size_t)B * 32, 256), 256, 0, s>>>(
        B, nout, M->loss_dim, M->loss_kern, M->loss_cut2, x, M->act.ptr + aoff[L],
        M->out_scale.ptr, M->out_shift.ptr, d, M->lossbuf.ptr);
  else
    k_mse<<<ceil_div((size_t)B * nout, 256), 256, 0, s>>>((size_t)B * nout, nout,
                                                          M->act.ptr + aoff[L], target,
                                                          M->out_scale.ptr, M->out_shift.ptr, d,
                                                          M->lossbuf.ptr);
  for (int l = L - 1; l >= 0; --l) {
    const int in = M->dims[l], out = M->dims[l + 1];
    if (l < L - 1)
      k_silu_back<<<ceil_div((size_t)B * out, 256), 256, 0, s>>>((size_t)B * out,
                                                                 M->pre.ptr + aoff[l + 1], d);
    float *gW = M->grads.ptr + M->woff[l];
    float *gb = M->grads.ptr + M->boff[l];
    // dW = X^T dZ  (in x out), db = colsum(dZ)
    gemm<true, false, 0, false>(s, in, out, (int)B, M->act.ptr + aoff[l], in, d, out, nullptr,
                                nullptr, gW, out);
    k_colsum<<<out, 256, 0, s>>>((int)B, out, d, gb);
    if (l > 0) {
      // dX = dZ W^T  (B x in)
      const float *W = M->params.ptr + M->woff[l];
      gemm<false, true, 0, false>(s, (int)B, in, out, d, out, W, out, nullptr, nullptr, dn, in);
      std::swap(d, dn);
    }
  }
  ABX_CHECK_CUDA(cudaGetLastError());
  if (loss) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(loss, M->lossbuf.ptr, sizeof(float), cudaMemcpyDeviceToHost, s));
    ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  }
  return ABX_OK;
}

int mlp_prepare_inference(abx_mlp *M) {
  if (M->infer_ready) return ABX_OK;
  ABX_REQUIRE(M->nlayers <= 8, ABX_ERR_INVALID, "too many layers for inference");
  M->wt_off.assign(M->nlayers, 0);
  M->in_pad.assign(M->nlayers, 0);
  size_t tot = 0;
  for (int l = 0; l < M->nlayers; ++l) {
    const int in = M->dims[l], out = M->dims[l + 1];
    ABX_REQUIRE(out % 8 == 0 && out <= IMAXW && in <= IMAXW, ABX_ERR_INVALID,
                "inference needs layer widths that are multiples of 8 and <= %d", IMAXW);
    M->in_pad[l] = (in + 15) / 16 * 16;
    M->wt_off[l] = tot;
    tot += (size_t)out * M->in_pad[l];
  }
  ABX_TRY(M->wt16.reserve(tot));
  for (int l = 0; l < M->nlayers; ++l) {
    const int in = M->dims[l], out = M->dims[l + 1];
    k_transpose_bf16<<<ceil_div((size_t)out * M->in_pad[l], 256), 256, 0, M->ctx->stream>>>(
        M->params.ptr + M->woff[l], in, out, M->in_pad[l], M->wt16.ptr + M->wt_off[l]);
  }
  ABX_CHECK_CUDA(cudaGetLastError());
  M->infer_ready = true;
  return ABX_OK;
}

}  // namespace

abx_context *mlp_context(const abx_mlp *M) { return M->ctx; }

int mlp_infer_bf16(abx_mlp *M, const float *x, int64_t n, float *y) {
  ABX_TRY(mlp_prepare_inference(M));
  if (n == 0) return ABX_OK;
  InferParams P{};
  P.nlayers = M->nlayers;
  for (int l = 0; l <= M->nlayers; ++l) P.dims[l] = M->dims[l];
  for (int l = 0; l < M->nlayers; ++l) {
    P.in_pad[l] = M->in_pad[l];
    P.wt[l] = M->wt16.ptr + M->wt_off[l];
    P.bias[l] = M->params.ptr + M->boff[l];
  }
  P.x = x;
  P.in_scale = M->in_scale;
  P.n = n;
  P.y = y;
  P.out_scale = M->out_scale.ptr;
  P.out_shift = M->out_shift.ptr;
  P.out_transform = M->out_transform;
  P.out_c = M->out_c;
  k_mlp_infer_bf16<<<ceil_div(n, IT), IW * 32, 0, M->ctx->stream>>>(P);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

int mlp_infer_fp32(abx_mlp *M, const float *x, int64_t n, float *y) {
  ABX_TRY(mlp_forward32(M, x, n));
  size_t o = 0;
  for (int l = 0; l < M->nlayers; ++l) o += (size_t)n * M->dims[l];
  const int nout = M->dims[M->nlayers];
  ABX_CHECK_CUDA(cudaMemcpyAsync(y, M->act.ptr + o, (size_t)n * nout * 4, cudaMemcpyDeviceToDevice,
                                 M->ctx->stream));
  k_denorm<<<ceil_div((size_t)n * nout, 256), 256, 0, M->ctx->stream>>>((size_t)n * nout, nout, y,
                                                                        M->out_scale.ptr,
                                                                        M->out_shift.ptr,
                                                                        M->out_transform, M->out_c);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

}  // namespace abx

using namespace abx;

extern "C" {

int abx_mlp_create(abx_context *ctx, int in_dim, int hidden, int nhidden, int out_dim,
                   uint64_t seed, abx_mlp **out) {
  ABX_REQUIRE(ctx && out, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(in_dim > 0 && hidden > 0 && nhidden >= 0 && out_dim > 0, ABX_ERR_INVALID,
              "invalid layer sizes");
  ABX_TRY(ctx_activate(ctx));
  abx_mlp *M = new abx_mlp();
  M->ctx = ctx;
  M->dims.push_back(in_dim);
  for (int i = 0; i < nhidden; ++i) M->dims.push_back(hidden);
  M->dims.push_back(out_dim);
  M->nlayers = (int)M->dims.size() - 1;
  size_t o = 0;
  for (int l = 0; l < M->nlayers; ++l) {
    M->woff.push_back(o);
    o += (size_t)M->dims[l] * M->dims[l + 1];
    M->boff.push_back(o);
    o += M->dims[l + 1];
  }
  M->nparams = o;
  int st;
  if ((st = M->params.reserve(o)) || (st = M->grads.reserve(o)) || (st = M->m1.reserve(o)) ||
      (st = M->m2.reserve(o)) || (st = M->out_scale.reserve(out_dim)) ||
      (st = M->out_shift.reserve(out_dim))) {
    delete M;
    return st;
  }
  cudaStream_t s = ctx->stream;
  cudaMemsetAsync(M->params.ptr, 0, o * 4, s);
  for (int l = 0; l < M->nlayers; ++l) {  // uniform(-a, a), a = sqrt(6 / (in + out))
    const int in = M->dims[l], ou = M->dims[l + 1];
    const float a = std::sqrt(6.0f / (float)(in + ou));
    k_init_uniform<<<ceil_div((size_t)in * ou, 256), 256, 0, s>>>(M->params.ptr + M->woff[l],
                                                                  (size_t)in * ou, a, seed + l);
  }
  cudaMemsetAsync(M->m1.ptr, 0, o * 4, s);
  cudaMemsetAsync(M->m2.ptr, 0, o * 4, s);
  std::vector<float> ones(out_dim, 1.0f), zeros(out_dim, 0.0f);
  cudaMemcpyAsync(M->out_scale.ptr, ones.data(), out_dim * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(M->out_shift.ptr, zeros.data(), out_dim * 4, cudaMemcpyHostToDevice, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    delete M;
    set_error("MLP initialisation failed");
    return ABX_ERR_CUDA;
  }
  ctx_retain(ctx);
  *out = M;
  return ABX_OK;
}

int abx_mlp_destroy(abx_mlp *M) {
  if (!M) return ABX_OK;
  abx_context *ctx = M->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete M;
  ctx_release(ctx);
  return ABX_OK;
}

int64_t abx_mlp_num_params(const abx_mlp *M) { return M ? (int64_t)M->nparams : -1; }

int abx_mlp_set_normalization(abx_mlp *M, float in_scale, const float *out_scale,
                              const float *out_shift) {
  ABX_REQUIRE(M && out_scale && out_shift, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(M->ctx));
  const int nout = M->dims.back();
  M->in_scale = in_scale;
  ABX_CHECK_CUDA(cudaMemcpy(M->out_scale.ptr, out_scale, nout * 4, cudaMemcpyDefault));
  ABX_CHECK_CUDA(cudaMemcpy(M->out_shift.ptr, out_shift, nout * 4, cudaMemcpyDefault));
  return ABX_OK;
}

int abx_mlp_set_output_transform(abx_mlp *M, int kind, float c) {
  ABX_REQUIRE(M && (kind == 0 || kind == 1) && c > 0, ABX_ERR_INVALID, "invalid transform");
  M->out_transform = kind;
  M->out_c = c;
  return ABX_OK;
}

int abx_mlp_set_loss(abx_mlp *M, int kind, int dim, const abx_kernel *k, double cutoff) {
  ABX_REQUIRE(M, ABX_ERR_INVALID, "null mlp");
  if (kind == ABX_LOSS_MSE) {
    M->loss_kind = kind;
    return ABX_OK;
  }
  ABX_REQUIRE(kind == ABX_LOSS_SPAI_RESIDUAL && k, ABX_ERR_INVALID, "unknown loss %d", kind);
  const int nout = M->dims.back();
  ABX_REQUIRE(dim >= 1 && dim <= 3 && nout <= 32 && M->dims[0] == nout * dim, ABX_ERR_INVALID,
              "residual loss needs out_dim <= 32 and in_dim = out_dim * dim (%d, %d, %d)",
              M->dims[0], nout, dim);
  ABX_REQUIRE(M->out_transform == 0, ABX_ERR_INVALID, "residual loss needs output transform 0");
  M->loss_kind = kind;
  M->loss_dim = dim;
  M->loss_kern = *k;
  M->loss_cut2 = cutoff > 0 ? (float)(cutoff * cutoff) : 0.f;
  return ABX_OK;
}

int abx_mlp_get_params(abx_mlp *M, float *out) {
  ABX_REQUIRE(M && out, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(M->ctx));
  ABX_CHECK_CUDA(cudaMemcpy(out, M->params.ptr, M->nparams * 4, cudaMemcpyDefault));
  return ABX_OK;
}

int abx_mlp_set_params(abx_mlp *M, const float *in) {
  ABX_REQUIRE(M && in, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(M->ctx));
  ABX_CHECK_CUDA(cudaMemcpy(M->params.ptr, in, M->nparams * 4, cudaMemcpyDefault));
  M->infer_ready = false;
  return ABX_OK;
}

int abx_mlp_gradients(abx_mlp *M, const float *x, const float *y, int64_t batch, float *grads,
                      float *loss) {
  ABX_REQUIRE(M && x && (y || M->loss_kind == ABX_LOSS_SPAI_RESIDUAL) && batch > 0,
              ABX_ERR_INVALID, "invalid argument");
  ABX_TRY(ctx_activate(M->ctx));
  const void *dx, *dy = nullptr;
  HostStage a, b;
  ABX_TRY(a.in(M->ctx, x, (size_t)batch * M->dims[0] * 4, &dx));
  if (y) ABX_TRY(b.in(M->ctx, y, (size_t)batch * M->dims.back() * 4, &dy));
  ABX_TRY(mlp_backward(M, (const float *)dx, (const float *)dy, batch, loss));
  if (grads) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(grads, M->grads.ptr, M->nparams * 4, cudaMemcpyDefault,
                                   M->ctx->stream));
    ABX_CHECK_CUDA(cudaStreamSynchronize(M->ctx->stream));
  }
  return ABX_OK;
}

int abx_mlp_train_step(abx_mlp *M, const float *x, const float *y, int64_t batch, float lr,
                       float *loss) {
  ABX_REQUIRE(M && x && (y || M->loss_kind == ABX_LOSS_SPAI_RESIDUAL) && batch > 0,
              ABX_ERR_INVALID, "invalid argument");
  ABX_TRY(ctx_activate(M->ctx));
  const void *dx, *dy = nullptr;
  ABX_TRY(M->sx.in(M->ctx, x, (size_t)batch * M->dims[0] * 4, &dx));
  if (y) ABX_TRY(M->sy.in(M->ctx, y, (size_t)batch * M->dims.back() * 4, &dy));
  ABX_TRY(mlp_backward(M, (const float *)dx, (const float *)dy, batch, loss));
  ++M->step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
  k_adam<<<ceil_div(M->nparams, 256), 256, 0, M->ctx->stream>>>(
      M->nparams, M->params.ptr, M->grads.ptr, M->m1.ptr, M->m2.ptr, lr, b1, b2, 1e-8f, c1, c2);
  ABX_CHECK_CUDA(cudaGetLastError());
  M->infer_ready = false;
  return ABX_OK;
}

int abx_mlp_forward(abx_mlp *M, const float *x, int64_t n, float *y, int precision) {
  ABX_REQUIRE(M && (n == 0 || (x && y)), ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(M->ctx));
  const void *dx;
  void *dy;
  HostStage a, b;
  const size_t ybytes = (size_t)n * M->dims.back() * 4;
  ABX_TRY(a.in(M->ctx, x, (size_t)n * M->dims[0] * 4, &dx));
  ABX_TRY(b.out(M->ctx, y, ybytes, &dy));
  if (precision == ABX_PREC_MIXED)
    ABX_TRY(mlp_infer_bf16(M, (const float *)dx, n, (float *)dy));
  else
    ABX_TRY(mlp_infer_fp32(M, (const float *)dx, n, (float *)dy));
  ABX_TRY(b.finish(M->ctx, y, ybytes));
  ABX_CHECK_CUDA(cudaStreamSynchronize(M->ctx->stream));
  return ABX_OK;
}

// File format (little-endian): "ABXMLP2\0", int32 nlayers, int32 dims[nlayers+1],
// float in_scale, int32 out_transform, float out_c, float out_scale[out],
// float out_shift[out], float params[].
int abx_mlp_save(abx_mlp *M, const char *path) {
  ABX_REQUIRE(M && path, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(M->ctx));
  const int nout = M->dims.back();
  std::vector<float> p(M->nparams), sc(nout), sh(nout);
  ABX_CHECK_CUDA(cudaMemcpy(p.data(), M->params.ptr, M->nparams * 4, cudaMemcpyDeviceToHost));
  ABX_CHECK_CUDA(cudaMemcpy(sc.data(), M->out_scale.ptr, nout * 4, cudaMemcpyDeviceToHost));
  ABX_CHECK_CUDA(cudaMemcpy(sh.data(), M->out_shift.ptr, nout * 4, cudaMemcpyDeviceToHost));
  FILE *f = fopen(path, "wb");
  ABX_REQUIRE(f, ABX_ERR_INVALID, "cannot open %s", path);
  const char magic[8] = {'A', 'B', 'X', 'M', 'L', 'P', '2', 0};
  fwrite(magic, 1, 8, f);
  const int32_t nl = M->nlayers;
  fwrite(&nl, 4, 1, f);
  for (int d : M->dims) {
    const int32_t v = d;
    fwrite(&v, 4, 1, f);
  }
  fwrite(&M->in_scale, 4, 1, f);
  const int32_t tr = M->out_transform;
  fwrite(&tr, 4, 1, f);
  fwrite(&M->out_c, 4, 1, f);
  fwrite(sc.data(), 4, nout, f);
  fwrite(sh.data(), 4, nout, f);
  fwrite(p.data(), 4, p.size(), f);
  fclose(f);
  return ABX_OK;
}

int abx_mlp_load(abx_context *ctx, const char *path, abx_mlp **out) {
  ABX_REQUIRE(ctx && path && out, ABX_ERR_INVALID, "null argument");
  FILE *f = fopen(path, "rb");
  ABX_REQUIRE(f, ABX_ERR_INVALID, "cannot open %s", path);
  char magic[8] = {};
  int32_t nl = 0;
  bool ok = fread(magic, 1, 8, f) == 8 && std::string(magic, 7) == "ABXMLP2" &&
            fread(&nl, 4, 1, f) == 1 && nl >= 1 && nl <= 16;
  std::vector<int32_t> dims(nl + 1);
  ok = ok && fread(dims.data(), 4, nl + 1, f) == (size_t)(nl + 1);
  if (!ok) {
    fclose(f);
    set_error("%s: not an MLP file", path);
    return ABX_ERR_INVALID;
  }
  for (int l = 1; l < nl; ++l)
    if (dims[l] != dims[1]) {
      fclose(f);
      set_error("%s: hidden layers must share one width", path);
      return ABX_ERR_INVALID;
    }
  abx_mlp *M = nullptr;
  int st = abx_mlp_create(ctx, dims[0], nl > 1 ? dims[1] : dims[nl], nl - 1, dims[nl], 0, &M);
  if (st != ABX_OK) {
    fclose(f);
    return st;
  }
  const int nout = dims[nl];
  std::vector<float> p(M->nparams), sc(nout), sh(nout);
  float in_scale = 1.f, oc = 1.f;
  int32_t tr = 0;
  ok = fread(&in_scale, 4, 1, f) == 1 && fread(&tr, 4, 1, f) == 1 && fread(&oc, 4, 1, f) == 1 &&
       fread(sc.data(), 4, nout, f) == (size_t)nout &&
       fread(sh.data(), 4, nout, f) == (size_t)nout &&
       fread(p.data(), 4, p.size(), f) == p.size();
  fclose(f);
  if (!ok) {
    abx_mlp_destroy(M);
    set_error("%s: truncated MLP file", path);
    return ABX_ERR_INVALID;
  }
  abx_mlp_set_params(M, p.data());
  abx_mlp_set_normalization(M, in_scale, sc.data(), sh.data());
  M->out_transform = tr;
  M->out_c = oc;
  *out = M;
  return ABX_OK;
}

}  // extern "C"
