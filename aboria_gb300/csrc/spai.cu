// Sparse approximate inverse preconditioner: x = M b with M stored as K
// (column index, value) pairs per row.  The rows come either from the exact
// local least-squares construction (spai_exact.cu) or from the learned model
// (mlp.cu); applying M is the same gather-multiply in both cases.
#include "common.cuh"
#include "handles.cuh"

namespace abx {

struct Spai {
  int64_t n = 0;
  int k = 0;
  DevBuf<int> cols;     // n*k, storage indices
  DevBuf<double> vals;  // n*k
};

namespace {
__global__ void k_spai_apply(const int *__restrict__ cols, const double *__restrict__ vals,
                             int64_t n, int k, const double *__restrict__ b,
                             double *__restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  const int *c = cols + i * k;
  const double *v = vals + i * k;
  for (int j = 0; j < k; ++j) s = fma(v[j], b[c[j]], s);
  x[i] = s;
}
}  // namespace

void spai_free(abx_precond *pc) {
  delete pc->spai;
  pc->spai = nullptr;
}

int spai_apply_device(abx_precond *pc, const double *b, double *x) {
  Spai *S = pc->spai;
  if (S->n == 0) return ABX_OK;
  k_spai_apply<<<ceil_div(S->n, 256), 256, 0, pc->ctx->stream>>>(S->cols.ptr, S->vals.ptr, S->n,
                                                                 S->k, b, x);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

}  // namespace abx

using namespace abx;

extern "C" int abx_precond_create_spai(abx_context *ctx, int64_t n, int k, const int32_t *cols,
                                       const double *vals, abx_precond **out) {
  ABX_REQUIRE(ctx && out && (n == 0 || (cols && vals)), ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(n >= 0 && k >= 1 && k <= 1024, ABX_ERR_INVALID, "invalid size");
  ABX_TRY(ctx_activate(ctx));
  Spai *S = new Spai();
  S->n = n;
  S->k = k;
  int st;
  if ((st = S->cols.reserve((size_t)n * k + 1)) || (st = S->vals.reserve((size_t)n * k + 1))) {
    delete S;
    return st;
  }
  if (n) {
    cudaMemcpyAsync(S->cols.ptr, cols, (size_t)n * k * 4, cudaMemcpyDefault, ctx->stream);
    cudaMemcpyAsync(S->vals.ptr, vals, (size_t)n * k * 8, cudaMemcpyDefault, ctx->stream);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
      delete S;
      set_error("copying the approximate inverse failed");
      return ABX_ERR_CUDA;
    }
  }
  abx_precond *pc = new abx_precond();
  pc->kind = 2;
  pc->spai = S;
  pc->ctx = ctx;
  pc->n = n;
  *out = pc;
  return ABX_OK;
}
