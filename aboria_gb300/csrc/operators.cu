// Kernel operators: create_sparse_operator / create_dense_operator and K*b.
//
// Reference: MatrixReplacement (src/Operators.h:75-281) with the Eigen product
// specialisation generic_product_impl::scaleAndAddTo
// (src/detail/Operators.h:207-229), which zero-initialises the destination and
// calls KernelX::evaluate.  The dense kernel restates KernelDense::evaluate
// (src/Kernels.h:212-239): for each row i, in column order j = 0..n-1,
// c_i += f(a_i, b_j) * b_j.  Each thread owns one row and walks the columns in
// exactly that order, so the FP64 mode reproduces the reference's summation
// order; columns are staged through shared memory 256 at a time.
#include <cmath>

#include "common.cuh"
#include "handles.cuh"

namespace abx {
namespace {

constexpr int DT = 256;  // rows per CTA = staged columns per tile

struct DenseParams {
  int dim, kind;
  double p0;
  float p0f, c_exp2;
  int64_t nr, nc;
  const double *rpos, *cpos;  // SoA storage order
  const double *b;
  const double *s_row, *s_col;
  double *c;
  double origin[3];
};

template <int KIND> __device__ __forceinline__ double dk64(double d2, double p0, double si,
                                                           double sj) {
  if (KIND == ABX_K_CONST) return p0;
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) return exp(-d2 * p0);
  if (KIND == ABX_K_WENDLAND_C2) {
    const double q = sqrt(d2) * p0;
    if (q >= 1.0) return 0.0;
    const double t = 1.0 - q;
    const double t2 = t * t;
    return t2 * t2 * (4.0 * q + 1.0);
  }
  if (KIND == ABX_K_LAPLACE) return 1.0 / (sqrt(d2) + p0);
  if (KIND == ABX_K_MULTIQUADRIC) return sqrt(d2 + p0);
  if (KIND == ABX_K_SCALAR_SUM) return si + sj;
  return 0.0;
}

// Hardware base-2 exponential (MUFU, ~2 ulp), flush-to-zero: the kernel
// weights it serves are negligible long before 2^-126.
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <int KIND> __device__ __forceinline__ float dk32(float d2, float p0f, float c_exp2) {
  if (KIND == ABX_K_CONST) return p0f;
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) return ex2_approx(d2 * c_exp2);
  if (KIND == ABX_K_WENDLAND_C2) {
    const float q = d2 * rsqrtf(fmaxf(d2, 1e-36f)) * p0f;
    const float t = fmaxf(1.0f - q, 0.0f);
    const float t2 = t * t;
    return t2 * t2 * fmaf(4.0f, q, 1.0f);
  }
  if (KIND == ABX_K_LAPLACE) return __fdividef(1.0f, d2 * rsqrtf(fmaxf(d2, 1e-36f)) + p0f);
  if (KIND == ABX_K_MULTIQUADRIC) {
    const float a = d2 + p0f;
    return a * rsqrtf(fmaxf(a, 1e-36f));
  }
  return 0.f;
}

template <int KIND> __global__ void __launch_bounds__(DT) k_dense_fp64(DenseParams P) {
  __shared__ double sx[DT], sy[DT], sz[DT], sb[DT], ss[DT];
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  const bool act = i < P.nr;
  double x0 = 0.0, x1 = 0.0, x2 = 0.0;
  if (act) {
    x0 = P.rpos[i];
    if (P.dim > 1) x1 = P.rpos[P.nr + i];
    if (P.dim > 2) x2 = P.rpos[2 * P.nr + i];
  }
  const double si = (KIND == ABX_K_SCALAR_SUM && act) ? P.s_row[i] : 0.0;
  double acc = 0.0;
  for (int64_t t = 0; t < P.nc; t += DT) {
    const int64_t j = t + threadIdx.x;
    if (j < P.nc) {
      sx[threadIdx.x] = P.cpos[j];
      sy[threadIdx.x] = P.dim > 1 ? P.cpos[P.nc + j] : 0.0;
      sz[threadIdx.x] = P.dim > 2 ? P.cpos[2 * P.nc + j] : 0.0;
      sb[threadIdx.x] = P.b[j];
      ss[threadIdx.x] = (KIND == ABX_K_SCALAR_SUM) ? P.s_col[j] : 0.0;
    }
    __syncthreads();
    const int nt = (int)((P.nc - t) < DT ? (P.nc - t) : DT);
    for (int jj = 0; jj < nt; ++jj) {
      // sum of squares in dimension order (0 + dx0^2 is exact)
      const double dx0 = __dsub_rn(sx[jj], x0);
      double d2 = __dmul_rn(dx0, dx0);
      if (P.dim > 1) {
        const double dx1 = __dsub_rn(sy[jj], x1);
        d2 = __dadd_rn(d2, __dmul_rn(dx1, dx1));
      }
      if (P.dim > 2) {
        const double dx2 = __dsub_rn(sz[jj], x2);
        d2 = __dadd_rn(d2, __dmul_rn(dx2, dx2));
      }
      acc = __dadd_rn(acc, __dmul_rn(dk64<KIND>(d2, P.p0, si, ss[jj]), sb[jj]));
    }
    __syncthreads();
  }
  if (act) P.c[i] = acc;
}

// Kernel values of two pairs: packed FP32x2 where the formula allows.
template <int KIND> __device__ __forceinline__ float2 dk32x2(float2 dd, float p0f, float c_exp2) {
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) {
    const float2 e = __fmul2_rn(dd, make_float2(c_exp2, c_exp2));
    return make_float2(ex2_approx(e.x), ex2_approx(e.y));
  }
  return make_float2(dk32<KIND>(dd.x, p0f, c_exp2), dk32<KIND>(dd.y, p0f, c_exp2));
}

// Mixed precision: FP32 offsets from the column domain centre, FP32 kernel
// values, one row per thread against two columns per packed FP32x2
// instruction; each staged tile of DT columns is summed in FP32 and tiles are
// added in FP64.  blockIdx.y selects a chunk of chunk_cols columns, so that
// small row counts still fill the GPU; with more than one chunk each CTA
// writes its row sums to partial[chunk][row] and k_dense_reduce adds the
// chunks in order (deterministic).  Columns are staged as pairs, pp[2h] = (x_a, x_b, y_a, y_b),
// pp[2h+1] = (z_a, z_b, b_a, b_b); an odd tail is paired with a far-away
// column of weight 0 (finite for every kernel).
template <int KIND>
__global__ void __launch_bounds__(DT) k_dense_mixed(DenseParams P, int64_t chunk_cols,
                                                    double *__restrict__ partial) {
  __shared__ float4 pp[DT];
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  const bool act = i < P.nr;
  float x0 = 0.f, x1 = 0.f, x2 = 0.f;
  if (act) {
    x0 = (float)(P.rpos[i] - P.origin[0]);
    if (P.dim > 1) x1 = (float)(P.rpos[P.nr + i] - P.origin[1]);
    if (P.dim > 2) x2 = (float)(P.rpos[2 * P.nr + i] - P.origin[2]);
  }
  const float2 nqx = make_float2(-x0, -x0), nqy = make_float2(-x1, -x1), nqz = make_float2(-x2, -x2);
  double acc = 0.0;
  const int64_t c0 = (int64_t)blockIdx.y * chunk_cols;
  const int64_t c1 = c0 + chunk_cols < P.nc ? c0 + chunk_cols : P.nc;
  for (int64_t t = c0; t < c1; t += DT) {
    const int64_t j = t + threadIdx.x;
    float x = 1e4f, y = 1e4f, z = 1e4f, w = 0.f;
    if (j < c1) {
      x = (float)(P.cpos[j] - P.origin[0]);
      y = P.dim > 1 ? (float)(P.cpos[P.nc + j] - P.origin[1]) : 0.f;
      z = P.dim > 2 ? (float)(P.cpos[2 * P.nc + j] - P.origin[2]) : 0.f;
      w = (float)P.b[j];
    }
    float *pf = reinterpret_cast<float *>(&pp[2 * (threadIdx.x >> 1)]);
    const int o = threadIdx.x & 1;
    pf[o] = x;
    pf[2 + o] = y;
    pf[4 + o] = z;
    pf[6 + o] = w;
    __syncthreads();
    const int nt = (int)((c1 - t) < DT ? (c1 - t) : DT);
    const int npair = (nt + 1) >> 1;
    float2 a2 = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int h = 0; h < npair; ++h) {
      const float4 A = pp[2 * h], B = pp[2 * h + 1];
      const float2 dx = __fadd2_rn(make_float2(A.x, A.y), nqx);
      const float2 dy = __fadd2_rn(make_float2(A.z, A.w), nqy);
      const float2 dz = __fadd2_rn(make_float2(B.x, B.y), nqz);
      float2 dd = __fmul2_rn(dx, dx);
      dd = __ffma2_rn(dy, dy, dd);
      dd = __ffma2_rn(dz, dz, dd);
      a2 = __ffma2_rn(dk32x2<KIND>(dd, P.p0f, P.c_exp2), make_float2(B.z, B.w), a2);
    }
    acc += (double)(a2.x + a2.y);
    __syncthreads();
  }
  if (act) {
    if (partial) partial[(int64_t)blockIdx.y * P.nr + i] = acc;
    else P.c[i] = acc;
  }
}

__global__ void k_dense_reduce(const double *__restrict__ partial, int64_t nr, int chunks,
                               double *__restrict__ c) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nr) return;
  double s = 0.0;
  for (int k = 0; k < chunks; ++k) s += partial[(int64_t)k * nr + i];
  c[i] = s;
}

template <int KIND>
int launch_dense(abx_context *ctx, const DenseParams &P, bool mixed, abx_operator *op) {
  const unsigned blocks = ceil_div(P.nr, DT);
  if (mixed && KIND != ABX_K_SCALAR_SUM) {
    // about 32 CTAs per SM in all: split the columns when the rows alone
    // give fewer
    const int64_t tiles = (P.nc + DT - 1) / DT;
    const int64_t want = (32 * (int64_t)std::max(ctx->num_sms, 1) + blocks - 1) / blocks;
    const int chunks = (int)std::max<int64_t>(1, std::min<int64_t>(want, std::min<int64_t>(tiles, 65535)));
    // no columns: one chunk that writes zeros
    const int64_t chunk_cols = tiles > 0 ? ((tiles + chunks - 1) / chunks) * DT : DT;
    const int used = tiles > 0 ? (int)((P.nc + chunk_cols - 1) / chunk_cols) : 1;
    double *partial = nullptr;
    if (used > 1) {
      ABX_TRY(op->partial.reserve((size_t)used * P.nr));
      partial = op->partial.ptr;
    }
    k_dense_mixed<KIND><<<dim3(blocks, std::max(used, 1)), DT, 0, ctx->stream>>>(P, chunk_cols,
                                                                               partial);
    if (partial)
      k_dense_reduce<<<ceil_div(P.nr, 256), 256, 0, ctx->stream>>>(partial, P.nr, used, P.c);
  } else
    k_dense_fp64<KIND><<<blocks, DT, 0, ctx->stream>>>(P);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

}  // namespace

int dense_matvec_device(abx_operator *op, const double *b, double *c) {
  abx_context *ctx = op->rows->ctx;
  DenseParams P{};
  P.dim = op->rows->dim;
  P.kind = op->k.kind;
  P.p0 = op->k.p[0];
  P.p0f = (float)op->k.p[0];
  P.c_exp2 = (float)(-op->k.p[0] * 1.4426950408889634);
  P.nr = op->rows->n;
  P.nc = op->cols->n;
  P.rpos = op->rows->pos.ptr;
  P.cpos = op->cols->pos.ptr;
  P.b = b;
  P.c = c;
  if (P.kind == ABX_K_SCALAR_SUM) {
    ABX_REQUIRE(op->rows->has_scalar && op->cols->has_scalar, ABX_ERR_STATE,
                "ABX_K_SCALAR_SUM needs a scalar column on both particle sets");
    P.s_row = op->rows->scalar.ptr;
    P.s_col = op->cols->scalar.ptr;
  }
  // FP32 coordinates are taken relative to the column domain centre when a
  // domain is set, else to the origin.
  for (int d = 0; d < 3; ++d) P.origin[d] = 0.0;
  if (op->cols->domain_set)
    for (int d = 0; d < P.dim; ++d)
      P.origin[d] = 0.5 * (op->cols->grid.lo[d] + op->cols->grid.hi[d]);
  if (P.nr == 0) return ABX_OK;
  const bool mixed = op->precision == ABX_PREC_MIXED;
  switch (P.kind) {
  case ABX_K_CONST: return launch_dense<ABX_K_CONST>(ctx, P, mixed, op);
  case ABX_K_GAUSSIAN: return launch_dense<ABX_K_GAUSSIAN>(ctx, P, mixed, op);
  case ABX_K_WENDLAND_C2: return launch_dense<ABX_K_WENDLAND_C2>(ctx, P, mixed, op);
  case ABX_K_COMPACT_GAUSSIAN: return launch_dense<ABX_K_COMPACT_GAUSSIAN>(ctx, P, mixed, op);
  case ABX_K_LAPLACE: return launch_dense<ABX_K_LAPLACE>(ctx, P, mixed, op);
  case ABX_K_MULTIQUADRIC: return launch_dense<ABX_K_MULTIQUADRIC>(ctx, P, mixed, op);
  case ABX_K_SCALAR_SUM: return launch_dense<ABX_K_SCALAR_SUM>(ctx, P, false, op);
  }
  set_error("unknown kernel kind %d", P.kind);
  return ABX_ERR_INVALID;
}

}  // namespace abx

using namespace abx;

extern "C" {

static int check_kernel(const abx_kernel *k) {
  ABX_REQUIRE(k, ABX_ERR_INVALID, "null kernel descriptor");
  ABX_REQUIRE(k->kind >= ABX_K_CONST && k->kind <= ABX_K_SCALAR_SUM, ABX_ERR_INVALID,
              "unknown kernel kind %d", k->kind);
  return ABX_OK;
}

int abx_create_sparse_operator(abx_particles *rows, abx_particles *cols, double radius,
                               const abx_kernel *k, abx_operator **out) {
  ABX_REQUIRE(rows && cols && out, ABX_ERR_INVALID, "null argument");
  ABX_TRY(check_kernel(k));
  ABX_REQUIRE(rows->ctx == cols->ctx, ABX_ERR_INVALID, "particle sets on different contexts");
  ABX_REQUIRE(rows->dim == cols->dim, ABX_ERR_INVALID, "dimension mismatch");
  ABX_REQUIRE(cols->searchable, ABX_ERR_STATE,
              "init_neighbour_search not called on the column particle set");
  ABX_REQUIRE(radius >= 0 && std::isfinite(radius), ABX_ERR_INVALID, "invalid radius");
  ABX_TRY(ctx_activate(rows->ctx));
  abx_operator *op = new abx_operator();
  op->kind = 0;
  op->rows = rows;
  op->cols = cols;
  op->radius = radius;
  op->k = *k;
  int st = pair_layout_build(op);
  if (st != ABX_OK) {
    if (op->pairs) pair_layout_free(op->pairs);
    delete op;
    return st;
  }
  particles_retain(rows);
  particles_retain(cols);
  *out = op;
  return ABX_OK;
}

int abx_create_dense_operator(abx_particles *rows, abx_particles *cols, const abx_kernel *k,
                              abx_operator **out) {
  ABX_REQUIRE(rows && cols && out, ABX_ERR_INVALID, "null argument");
  ABX_TRY(check_kernel(k));
  ABX_REQUIRE(rows->ctx == cols->ctx, ABX_ERR_INVALID, "particle sets on different contexts");
  ABX_REQUIRE(rows->dim == cols->dim, ABX_ERR_INVALID, "dimension mismatch");
  abx_operator *op = new abx_operator();
  op->kind = 1;
  op->rows = rows;
  op->cols = cols;
  op->k = *k;
  particles_retain(rows);
  particles_retain(cols);
  *out = op;
  return ABX_OK;
}

int abx_operator_destroy(abx_operator *op) {
  if (!op) return ABX_OK;
  abx_particles *rows = op->rows, *cols = op->cols;
  cudaSetDevice(rows->ctx->device);
  cudaStreamSynchronize(rows->ctx->stream);
  if (op->pairs) pair_layout_free(op->pairs);
  if (op->fmm) fmm_plan_free(op->fmm);
  delete op;
  particles_release(rows);
  particles_release(cols);
  return ABX_OK;
}

int abx_operator_set_precision(abx_operator *op, int mode) {
  ABX_REQUIRE(op, ABX_ERR_INVALID, "null operator");
  ABX_REQUIRE(mode == ABX_PREC_FP64 || mode == ABX_PREC_MIXED, ABX_ERR_INVALID,
              "unknown precision mode %d", mode);
  op->precision = mode;
  return ABX_OK;
}

int64_t abx_operator_rows(const abx_operator *op) { return op ? op->rows->n : -1; }
int64_t abx_operator_cols(const abx_operator *op) { return op ? op->cols->n : -1; }

int abx_operator_matvec(abx_operator *op, const double *b, double *c) {
  ABX_REQUIRE(op, ABX_ERR_INVALID, "null operator");
  const int64_t nr = op->rows->n, nc = op->cols->n;
  ABX_REQUIRE((b || nc == 0) && (c || nr == 0), ABX_ERR_INVALID, "null vector");
  abx_context *ctx = op->rows->ctx;
  ABX_TRY(ctx_activate(ctx));
  if (op->kind == 0)
    ABX_REQUIRE(op->cols->searchable, ABX_ERR_STATE,
                "init_neighbour_search not called on the column particle set");
  const void *bd;
  void *cd;
  ABX_TRY(op->stage_b.in(ctx, b, (size_t)nc * sizeof(double), &bd));
  ABX_TRY(op->stage_c.out(ctx, c, (size_t)nr * sizeof(double), &cd));
  if (op->kind == 0)
    ABX_TRY(sparse_matvec_device(op, (const double *)bd, (double *)cd));
  else if (op->kind == 1)
    ABX_TRY(dense_matvec_device(op, (const double *)bd, (double *)cd));
  else
    ABX_TRY(fmm_matvec_device(op, (const double *)bd, (double *)cd));
  ABX_TRY(op->stage_c.finish(ctx, c, (size_t)nr * sizeof(double)));
  return ABX_OK;
}

int abx_operator_last_stats(abx_operator *op, int64_t *candidates, int64_t *pairs) {
  ABX_REQUIRE(op, ABX_ERR_INVALID, "null operator");
  if (candidates) *candidates = op->last_candidates;
  if (pairs) *pairs = op->last_pairs;
  return ABX_OK;
}

}  // extern "C"
