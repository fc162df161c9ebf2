// Sparse approximate inverse preconditioner: x = M b with M stored as K
// (column index, value) pairs per row.  The rows come either from the exact
// local least-squares construction (spai_exact.cu) or from the learned model
// (mlp.cu); applying M is the same gather-multiply in both cases.
#include <chrono>

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
  ctx_retain(ctx);
  *out = pc;
  return ABX_OK;
}

// ---------------------------------------------------------------------------
// Exact local least-squares rows: CardinalFunctionsPreconditioner::factorize
// (src/Preconditioners.h:1025-1082) restricted to a k-nearest-neighbour
// support.  For row i with support S (its k nearest neighbours, i first), the
// weights solve min_w || A(S,:)^T w - e_i ||_2 over all columns; only columns
// in U = union of the kernel neighbourhoods of S carry non-zeros, so the
// problem is the |U| x k system B w = e_i with B(u,s) = coeff(s, u)
// (strict |dx| < r, periodic-corrected dx).  It is solved by Householder QR
// with column pivoting (the reference calls colPivHouseholderQr).
//
// One CTA per row (persistent grid): U is collected in a shared-memory hash
// set, B lives in a per-CTA global scratch slot (column-major), the QR steps
// are warp-per-column reductions, the 32x32 back substitution is serial.
namespace abx {
namespace {

constexpr int LS_T = 256;
constexpr int LS_HT = 8192;   // hash slots
constexpr int LS_MCAP = 3072; // max |U|
constexpr int LS_K = 32;
constexpr int LS_LOCAL_T = 256;  // local mode: 8 rows (warps) per block

struct LsParams {
  int dim, kind;
  double p0, r2;
  double L[3];
  int periodic[3];
  const double *pos;  // SoA storage order
  int64_t n;
  const int64_t *rowptr;
  const int32_t *cols;
  const int32_t *knn;  // n * k
  int k;
  double *scratch;     // gridDim.x * LS_MCAP * LS_K
  double *vals;        // n * k
  int *counter;
  int *status;         // 0 ok; 1 |U| over capacity
  int local;           // 1: U = S (row of the local block inverse)
  const int32_t *subset;  // rows to solve (null: all n rows)
  int64_t nrows;          // rows to solve
};

template <int KIND> __device__ __forceinline__ double ls_coeff(const LsParams &P, int a, int b) {
  double d2 = 0.0;
  for (int d = 0; d < P.dim; ++d) {
    double dx = __dsub_rn(P.pos[(int64_t)d * P.n + b], P.pos[(int64_t)d * P.n + a]);
    if (P.periodic[d]) {
      const double w = P.L[d];
      while (dx > w / 2) dx -= w;
      while (dx <= -w / 2) dx += w;
    }
    d2 = __dadd_rn(d2, __dmul_rn(dx, dx));
  }
  if (!(d2 < P.r2)) return 0.0;
  if (KIND == ABX_K_CONST) return P.p0;
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) return exp(-d2 * P.p0);
  if (KIND == ABX_K_WENDLAND_C2) {
    const double q = sqrt(d2) * P.p0;
    if (q >= 1.0) return 0.0;
    const double t = 1.0 - q;
    return t * t * t * t * (4.0 * q + 1.0);
  }
  if (KIND == ABX_K_LAPLACE) return 1.0 / (sqrt(d2) + P.p0);
  if (KIND == ABX_K_MULTIQUADRIC) return sqrt(d2 + P.p0);
  return 0.0;
}

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < LS_T / 32; ++i) t += red[i];
  return t;
}

constexpr size_t LS_SMEM = (size_t)LS_MCAP * 2 * sizeof(double) + (size_t)LS_HT * sizeof(int) +
                           (size_t)LS_MCAP * sizeof(int);

template <int KIND> __global__ void __launch_bounds__(LS_T) k_spai_ls(LsParams P) {
  extern __shared__ __align__(16) unsigned char ls_smem[];
  double *e = (double *)ls_smem;
  double *v = e + LS_MCAP;
  int *hset = (int *)(v + LS_MCAP);
  int *U = hset + LS_HT;
  __shared__ double red[LS_T / 32];
  __shared__ double cn[LS_K];
  __shared__ int S[LS_K], perm[LS_K];
  __shared__ int s_m, s_row, s_pi, s_rank;
  __shared__ double s_alpha;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k = P.k;
  double *B = P.scratch + (size_t)blockIdx.x * LS_MCAP * LS_K;
  for (;;) {
    if (tid == 0) s_row = atomicAdd(P.counter, 1);
    __syncthreads();
    if (s_row >= P.nrows) break;
    const int i = P.subset ? P.subset[s_row] : s_row;
    for (int h = tid; h < LS_HT; h += LS_T) hset[h] = -1;
    if (tid < k) {
      S[tid] = P.knn[(int64_t)i * k + tid];
      perm[tid] = tid;
    }
    if (tid == 0) s_m = 0;
    __syncthreads();
    if (P.local) {  // square local system: U = S
      if (tid < k) U[tid] = S[tid] >= 0 ? S[tid] : -1 - tid;
      if (tid == 0) s_m = k;
    }
    // U: union of the support's kernel neighbourhoods (hash set)
    for (int s = 0; s < k && !P.local; ++s) {
      const int a = S[s];
      if (a < 0) continue;
      for (int64_t t = P.rowptr[a] + tid; t < P.rowptr[a + 1]; t += LS_T) {
        const int c = P.cols[t];
        unsigned hsh = ((unsigned)c * 2654435761u) & (LS_HT - 1);
        for (int probe = 0; probe < LS_HT; ++probe) {
          const int old = atomicCAS(&hset[hsh], -1, c);
          if (old == -1) {
            const int slot = atomicAdd(&s_m, 1);
            if (slot < LS_MCAP) U[slot] = c;
            break;
          }
          if (old == c) break;
          hsh = (hsh + 1) & (LS_HT - 1);
        }
      }
    }
    __syncthreads();
    const int m = s_m;
    if (m > LS_MCAP) {
      if (tid == 0) atomicExch(P.status, 1);
      __syncthreads();
      continue;
    }
    // B(u, s) = coeff(S[s], U[u]); rhs e = e_i
    for (int64_t t = tid; t < (int64_t)m * k; t += LS_T) {
      const int s = (int)(t / m), u = (int)(t % m);
      B[(size_t)s * LS_MCAP + u] = (S[s] >= 0 && U[u] >= 0) ? ls_coeff<KIND>(P, S[s], U[u]) : 0.0;
    }
    for (int u = tid; u < m; u += LS_T) {
      e[u] = (U[u] == i) ? 1.0 : 0.0;
      if (U[u] == i) s_pi = u;
    }
    if (tid == 0) s_rank = k;
    __syncthreads();
    double r00 = 0.0;
    for (int j = 0; j < k; ++j) {
      // squared norms of the remaining columns over rows j..m-1
      for (int c = j + warp; c < k; c += LS_T / 32) {
        double sacc = 0.0;
        for (int u = j + lane; u < m; u += 32) {
          const double b = B[(size_t)c * LS_MCAP + u];
          sacc = fma(b, b, sacc);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
        if (lane == 0) cn[c] = sacc;
      }
      __syncthreads();
      if (tid == 0) {
        int p = j;
        for (int c = j + 1; c < k; ++c)
          if (cn[c] > cn[p]) p = c;
        red[0] = (double)p;
      }
      __syncthreads();
      const int p = (int)red[0];
      __syncthreads();
      if (p != j) {
        for (int u = tid; u < m; u += LS_T) {
          const double t = B[(size_t)j * LS_MCAP + u];
          B[(size_t)j * LS_MCAP + u] = B[(size_t)p * LS_MCAP + u];
          B[(size_t)p * LS_MCAP + u] = t;
        }
        if (tid == 0) {
          const int t = perm[j];
          perm[j] = perm[p];
          perm[p] = t;
          const double c = cn[j];
          cn[j] = cn[p];
          cn[p] = c;
        }
      }
      __syncthreads();
      const double nrm = sqrt(cn[j]);
      if (j == 0) r00 = nrm;
      if (nrm <= 1e-13 * r00 || nrm == 0.0 || j >= m) {
        if (tid == 0) s_rank = j;
        __syncthreads();
        break;
      }
      // Householder vector v = x - alpha e1, alpha = -sign(x0) |x|
      const double x0 = B[(size_t)j * LS_MCAP + j];
      const double alpha = x0 > 0 ? -nrm : nrm;
      for (int u = j + tid; u < m; u += LS_T) v[u] = B[(size_t)j * LS_MCAP + u];
      __syncthreads();
      if (tid == 0) {
        v[j] = x0 - alpha;
        s_alpha = alpha;
      }
      __syncthreads();
      double vv = 0.0;
      for (int u = j + tid; u < m; u += LS_T) vv = fma(v[u], v[u], vv);
      vv = block_sum(vv, red);
      const double tau = vv > 0 ? 2.0 / vv : 0.0;
      // apply to columns j+1..k-1 (warp per column) and to e
      for (int c = j + 1 + warp; c < k; c += LS_T / 32) {
        double sacc = 0.0;
        for (int u = j + lane; u < m; u += 32) sacc = fma(v[u], B[(size_t)c * LS_MCAP + u], sacc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
        const double f = tau * sacc;
        for (int u = j + lane; u < m; u += 32) B[(size_t)c * LS_MCAP + u] -= f * v[u];
      }
      double se = 0.0;
      for (int u = j + tid; u < m; u += LS_T) se = fma(v[u], e[u], se);
      se = block_sum(se, red);
      for (int u = j + tid; u < m; u += LS_T) e[u] -= tau * se * v[u];
      __syncthreads();
      if (tid == 0) B[(size_t)j * LS_MCAP + j] = s_alpha;
      __syncthreads();
    }
    __syncthreads();
    if (tid == 0) {
      const int rk = s_rank;
      double w[LS_K];
      for (int j = k - 1; j >= 0; --j) {
        if (j >= rk) {
          w[j] = 0.0;
          continue;
        }
        double t = e[j];
        for (int c = j + 1; c < rk; ++c) t -= B[(size_t)c * LS_MCAP + j] * w[c];
        w[j] = t / B[(size_t)j * LS_MCAP + j];
      }
      for (int j = 0; j < k; ++j) P.vals[(int64_t)i * k + perm[j]] = w[j];
    }
    __syncthreads();
  }
}

// Local mode (U = S, the k x k system of the row's support) with one warp
// per row: lane c holds column c of B, B(u, c) = coeff(S[c], S[u]), in
// registers, and lane u the rhs entry e_u.  The same Householder QR with
// column pivoting as k_spai_ls (pivot: the first column of largest norm over
// the remaining rows; stop at a norm <= 1e-13 |R00|), then the back
// substitution over the rank; the Householder vector passes through a
// per-warp shared-memory row.
template <int KIND> __global__ void __launch_bounds__(LS_LOCAL_T) k_spai_local(LsParams P) {
  constexpr int WPB = LS_LOCAL_T / 32;
  __shared__ double vsh[WPB][LS_K];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int k = P.k;
  double *v = vsh[wib];
  for (int64_t r = (int64_t)blockIdx.x * WPB + wib; r < P.nrows; r += (int64_t)gridDim.x * WPB) {
    const int64_t i = P.subset ? P.subset[r] : r;
    const int s = lane < k ? P.knn[i * k + lane] : -1;
    double col[LS_K];
#pragma unroll
    for (int u = 0; u < LS_K; ++u) {
      const int su = __shfl_sync(0xffffffffu, s, u);
      col[u] = (s >= 0 && su >= 0) ? ls_coeff<KIND>(P, s, su) : 0.0;
    }
    double eu = (s >= 0 && s == i) ? 1.0 : 0.0;
    int perm = lane;
    int rank = k;
    double r00 = 0.0;
    for (int j = 0; j < k; ++j) {
      // norms of the remaining columns over rows j..k-1
      double cn = 0.0;
#pragma unroll
      for (int u = 0; u < LS_K; ++u)
        if (u >= j) cn = fma(col[u], col[u], cn);
      double bv = (lane >= j && lane < k) ? cn : -1.0;
      int bl = lane;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int ol = __shfl_xor_sync(0xffffffffu, bl, o);
        if (ov > bv || (ov == bv && ol < bl)) {
          bv = ov;
          bl = ol;
        }
      }
      const int p = bl;
      if (p != j) {  // swap columns j and p (and their permutation entries)
        const int src = lane == j ? p : (lane == p ? j : lane);
#pragma unroll
        for (int u = 0; u < LS_K; ++u) col[u] = __shfl_sync(0xffffffffu, col[u], src);
        perm = __shfl_sync(0xffffffffu, perm, src);
      }
      const double nrm = sqrt(bv);
      if (j == 0) r00 = nrm;
      if (nrm <= 1e-13 * r00 || nrm == 0.0) {
        rank = j;
        break;
      }
      // Householder vector of column j (rows j..k-1): v = x - alpha e_j
      if (lane == j) {
#pragma unroll
        for (int u = 0; u < LS_K; ++u) v[u] = u >= j ? col[u] : 0.0;
      }
      __syncwarp();
      const double x0 = v[j];
      const double alpha = x0 > 0 ? -nrm : nrm;
      __syncwarp();
      if (lane == 0) v[j] = x0 - alpha;
      __syncwarp();
      double vv = 0.0;
#pragma unroll
      for (int u = 0; u < LS_K; ++u)
        if (u >= j) vv = fma(v[u], v[u], vv);
      const double tau = vv > 0 ? 2.0 / vv : 0.0;
      // apply to the columns j+1..k-1 and to e
      if (lane > j && lane < k) {
        double d = 0.0;
#pragma unroll
        for (int u = 0; u < LS_K; ++u)
          if (u >= j) d = fma(v[u], col[u], d);
        const double f = tau * d;
#pragma unroll
        for (int u = 0; u < LS_K; ++u)
          if (u >= j) col[u] = fma(-f, v[u], col[u]);
      }
      double se = lane >= j ? v[lane] * eu : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
      if (lane >= j) eu = fma(-tau * se, v[lane], eu);
      if (lane == j) {
#pragma unroll
        for (int u = 0; u < LS_K; ++u)
          if (u == j) col[u] = alpha;
      }
      __syncwarp();
    }
    // back substitution R w = (Q^T e) over the first `rank` columns: lane c
    // holds R(0..c, c) in col[0..c], lane j holds (Q^T e)_j in eu
    double w = 0.0;
    for (int j = rank - 1; j >= 0; --j) {
      double rjc = 0.0;
#pragma unroll
      for (int u = 0; u < LS_K; ++u)
        if (u == j) rjc = col[u];
      double t = (lane > j && lane < rank) ? rjc * w : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      const double ej = __shfl_sync(0xffffffffu, eu, j);
      if (lane == j) w = (ej - t) / rjc;
    }
    if (lane < k) P.vals[i * k + perm] = lane < rank ? w : 0.0;
  }
}

}  // namespace

// Exact least-squares SPAI rows for the sparse operator `op` (rows == cols)
// on the k-nearest-neighbour support; outputs device arrays cols (n*k) and
// vals (n*k) in storage order.
int self_csr_device(abx_particles *p, double r, DevBuf<int64_t> &rowptr, DevBuf<int32_t> &cols,
                    int64_t &nnz);
int knn_device(abx_particles *p, int k, int32_t *idx, double *d2);

namespace {
// Events at the boundaries of the learned preconditioner's set-up phases.
// Timing is best effort: if an event cannot be created the phases read 0.
struct PhaseEvents {
  cudaStream_t s;
  cudaEvent_t e[5] = {};
  bool ok = true;
  explicit PhaseEvents(cudaStream_t st) : s(st) {
    for (auto &x : e) ok = ok && cudaEventCreate(&x) == cudaSuccess;
  }
  ~PhaseEvents() {
    for (auto &x : e)
      if (x) cudaEventDestroy(x);
  }
  void mark(int i) {
    if (ok) ok = cudaEventRecord(e[i], s) == cudaSuccess;
  }
  // once mark(4) has been recorded
  void elapsed(double out[4]) {
    if (ok) ok = cudaEventSynchronize(e[4]) == cudaSuccess;
    for (int i = 0; i < 4; ++i) {
      float ms = 0.0f;
      const bool got = ok && cudaEventElapsedTime(&ms, e[i], e[i + 1]) == cudaSuccess;
      if (ok && !got) cudaGetLastError();  // the timing's own error, not the caller's
      out[i] = got ? 1e-3 * ms : 0.0;
    }
  }
};
}  // namespace

// subset (device, nsub rows) restricts the solve to those rows; knn_given
// says cols_out already holds the k-nearest-neighbour supports.
int spai_exact_rows(abx_operator *op, int k, int32_t *cols_out, double *vals_out, int local,
                    const int32_t *subset = nullptr, int64_t nsub = -1, bool knn_given = false) {
  abx_particles *p = op->rows;
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  ABX_REQUIRE(op->kind == 0 && op->rows == op->cols, ABX_ERR_INVALID,
              "SPAI rows need a square sparse operator (rows == cols)");
  ABX_REQUIRE(k >= 1 && k <= LS_K, ABX_ERR_INVALID, "k must be in 1..%d", LS_K);
  ABX_REQUIRE(op->k.kind != ABX_K_SCALAR_SUM, ABX_ERR_INVALID, "kernel not supported");
  const int64_t n = p->n;
  if (n == 0) return ABX_OK;
  if (!knn_given) ABX_TRY(knn_device(p, k, cols_out, nullptr));
  const int64_t nrows = subset ? nsub : n;
  if (nrows == 0) return ABX_OK;
  DevBuf<int64_t> rowptr;
  DevBuf<int32_t> cols;
  int64_t nnz = 0;
  if (!local) ABX_TRY(self_csr_device(p, op->radius, rowptr, cols, nnz));
  const int grid = (int)std::min<int64_t>(nrows, (int64_t)ctx->num_sms * 2);
  DevBuf<double> scratch;
  DevBuf<int> flags;
  if (!local) ABX_TRY(scratch.reserve((size_t)grid * LS_MCAP * LS_K));
  ABX_TRY(flags.reserve(2));
  ABX_CHECK_CUDA(cudaMemsetAsync(flags.ptr, 0, 2 * sizeof(int), s));
  LsParams P{};
  P.dim = p->dim;
  P.kind = op->k.kind;
  P.p0 = op->k.p[0];
  P.r2 = op->radius * op->radius;
  for (int d = 0; d < 3; ++d) {
    P.L[d] = p->grid.hi[d] - p->grid.lo[d];
    P.periodic[d] = d < p->dim ? p->grid.periodic[d] : 0;
  }
  P.pos = p->pos.ptr;
  P.n = n;
  P.rowptr = rowptr.ptr;
  P.cols = cols.ptr;
  P.knn = cols_out;
  P.k = k;
  P.scratch = scratch.ptr;
  P.vals = vals_out;
  P.counter = flags.ptr;
  P.status = flags.ptr + 1;
  P.local = local;
  P.subset = subset;
  P.nrows = nrows;
  auto launch = [&](auto kern) -> int {
    ABX_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)LS_SMEM));
    kern<<<grid, LS_T, LS_SMEM, s>>>(P);
    return ABX_OK;
  };
  // local mode: a warp per row, every SM kept full
  const int lgrid = (int)std::min<int64_t>((nrows + LS_LOCAL_T / 32 - 1) / (LS_LOCAL_T / 32),
                                           (int64_t)ctx->num_sms * 8);
  auto launch_local = [&](auto kern) -> int {
    kern<<<lgrid, LS_LOCAL_T, 0, s>>>(P);
    return ABX_OK;
  };
  if (local) {
    switch (P.kind) {
    case ABX_K_CONST: ABX_TRY(launch_local(k_spai_local<ABX_K_CONST>)); break;
    case ABX_K_GAUSSIAN: ABX_TRY(launch_local(k_spai_local<ABX_K_GAUSSIAN>)); break;
    case ABX_K_WENDLAND_C2: ABX_TRY(launch_local(k_spai_local<ABX_K_WENDLAND_C2>)); break;
    case ABX_K_COMPACT_GAUSSIAN: ABX_TRY(launch_local(k_spai_local<ABX_K_COMPACT_GAUSSIAN>)); break;
    case ABX_K_LAPLACE: ABX_TRY(launch_local(k_spai_local<ABX_K_LAPLACE>)); break;
    case ABX_K_MULTIQUADRIC: ABX_TRY(launch_local(k_spai_local<ABX_K_MULTIQUADRIC>)); break;
    }
  } else {
    switch (P.kind) {
    case ABX_K_CONST: ABX_TRY(launch(k_spai_ls<ABX_K_CONST>)); break;
    case ABX_K_GAUSSIAN: ABX_TRY(launch(k_spai_ls<ABX_K_GAUSSIAN>)); break;
    case ABX_K_WENDLAND_C2: ABX_TRY(launch(k_spai_ls<ABX_K_WENDLAND_C2>)); break;
    case ABX_K_COMPACT_GAUSSIAN: ABX_TRY(launch(k_spai_ls<ABX_K_COMPACT_GAUSSIAN>)); break;
    case ABX_K_LAPLACE: ABX_TRY(launch(k_spai_ls<ABX_K_LAPLACE>)); break;
    case ABX_K_MULTIQUADRIC: ABX_TRY(launch(k_spai_ls<ABX_K_MULTIQUADRIC>)); break;
    }
  }
  ABX_CHECK_CUDA(cudaGetLastError());
  int st[2];
  ABX_CHECK_CUDA(cudaMemcpyAsync(st, flags.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  ABX_REQUIRE(st[1] == 0, ABX_ERR_CAPACITY,
              "SPAI least squares: a row's column set exceeds %d entries", LS_MCAP);
  return ABX_OK;
}

}  // namespace abx

extern "C" int abx_spai_exact_rows(abx_operator *op, int k, int32_t *cols, double *vals) {
  ABX_REQUIRE(op && cols && vals, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(op->rows->ctx));
  const int64_t n = op->rows->n;
  HostStage sc, sv;
  void *dc, *dv;
  ABX_TRY(sc.out(op->rows->ctx, cols, (size_t)n * k * 4, &dc));
  ABX_TRY(sv.out(op->rows->ctx, vals, (size_t)n * k * 8, &dv));
  ABX_TRY(spai_exact_rows(op, k, (int32_t *)dc, (double *)dv, 0));
  ABX_TRY(sc.finish(op->rows->ctx, cols, (size_t)n * k * 4));
  ABX_TRY(sv.finish(op->rows->ctx, vals, (size_t)n * k * 8));
  return ABX_OK;
}

// ---------------------------------------------------------------------------
// Learned approximate inverse: features -> MLP (BF16 tensor cores) -> weights.
namespace abx {
int mlp_infer_bf16(abx_mlp *M, const float *x, int64_t n, float *y);
int mlp_infer_fp32(abx_mlp *M, const float *x, int64_t n, float *y);
abx_context *mlp_context(const abx_mlp *M);

// Work queued on `to` after this call waits for everything queued on `from`.
static int stream_order(cudaStream_t from, cudaStream_t to) {
  if (from == to) return ABX_OK;
  cudaEvent_t e;
  ABX_CHECK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaError_t r = cudaEventRecord(e, from);
  if (r == cudaSuccess) r = cudaStreamWaitEvent(to, e, 0);
  cudaEventDestroy(e);  // released once the recorded work completes
  if (r != cudaSuccess) {
    set_error("stream ordering: %s", cudaGetErrorString(r));
    return ABX_ERR_CUDA;
  }
  return ABX_OK;
}

namespace {
// feats[i][j*D + d] = eps * (x_{S_ij} - x_i)_d with periodic minimum image.
__global__ void k_spai_features(const double *__restrict__ pos, int64_t n, int dim,
                                const int32_t *__restrict__ knn, int k, double eps, GridDesc g,
                                float *__restrict__ feats) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * k) return;
  const int64_t i = t / k;  // row; t % k is the support slot
  const int s = knn[t];
  for (int d = 0; d < dim; ++d) {
    double dx = s >= 0 ? pos[(int64_t)d * n + s] - pos[(int64_t)d * n + i] : 0.0;
    if (g.periodic[d]) {
      const double w = g.hi[d] - g.lo[d];
      while (dx > w / 2) dx -= w;
      while (dx <= -w / 2) dx += w;
    }
    feats[t * dim + d] = (float)(eps * dx);
  }
}

// Rows whose nearest other support point (k-NN entry 1) has kernel value
// phi > exact_phi: their approximate-inverse row is solved exactly.
__global__ void k_flag_close(const double *__restrict__ d2, int64_t n, int k, int kind, double p0,
                             double exact_phi, int32_t *__restrict__ list,
                             int *__restrict__ count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || k < 2) return;
  const double r2 = d2[i * k + 1];
  double phi = 0.0;
  switch (kind) {
  case ABX_K_GAUSSIAN:
  case ABX_K_COMPACT_GAUSSIAN: phi = exp(-p0 * r2); break;
  case ABX_K_WENDLAND_C2: {
    const double q = sqrt(r2) * p0;
    const double t = q < 1.0 ? 1.0 - q : 0.0;
    phi = t * t * t * t * (4.0 * q + 1.0);
    break;
  }
  default: phi = 1.0;  // kernels not normalised to phi(0) = 1: every row exact
  }
  if (phi > exact_phi) list[atomicAdd(count, 1)] = (int32_t)i;
}

__global__ void k_f2d_masked(const float *__restrict__ y, const int32_t *__restrict__ cols,
                             int64_t n, double *__restrict__ vals) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) vals[i] = cols[i] >= 0 ? (double)y[i] : 0.0;
}
}  // namespace

int knn_device(abx_particles *p, int k, int32_t *idx, double *d2);


int spai_features_device(abx_particles *p, const int32_t *knn, int k, double eps, float *feats) {
  const int64_t n = p->n;
  if (n == 0) return ABX_OK;
  k_spai_features<<<ceil_div((size_t)n * k, 256), 256, 0, p->ctx->stream>>>(
      p->pos.ptr, n, p->dim, knn, k, eps, p->grid, feats);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}

}  // namespace abx

extern "C" int abx_spai_features(abx_particles *p, const int32_t *knn, int k, double eps,
                                 float *feats) {
  ABX_REQUIRE(p && (p->n == 0 || (knn && feats)), ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(p->ctx));
  const int64_t n = p->n;
  HostStage a, b;
  const void *dk;
  void *df;
  ABX_TRY(a.in(p->ctx, knn, (size_t)n * k * 4, &dk));
  ABX_TRY(b.out(p->ctx, feats, (size_t)n * k * p->dim * 4, &df));
  ABX_TRY(spai_features_device(p, (const int32_t *)dk, k, eps, (float *)df));
  ABX_TRY(b.finish(p->ctx, feats, (size_t)n * k * p->dim * 4));
  ABX_CHECK_CUDA(cudaStreamSynchronize(p->ctx->stream));
  return ABX_OK;
}

extern "C" int abx_precond_create_learned(abx_operator *op, abx_mlp *mlp, double eps, int k,
                                          int precision, double exact_phi, abx_precond **out) {
  ABX_REQUIRE(op && mlp && out, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(op->rows == op->cols, ABX_ERR_INVALID, "needs a square operator");
  abx_particles *p = op->rows;
  ABX_REQUIRE(p->searchable, ABX_ERR_STATE, "init_neighbour_search not called");
  ABX_REQUIRE(k >= 1 && k <= 64, ABX_ERR_INVALID, "k must be in 1..64");
  ABX_REQUIRE(mlp_context(mlp)->device == p->ctx->device, ABX_ERR_INVALID,
              "the model and the operator must be on one device");
  ABX_TRY(ctx_activate(p->ctx));
  const int64_t n = p->n;
  abx_precond *pc = new abx_precond();
  pc->kind = 2;
  pc->ctx = p->ctx;
  pc->n = n;
  pc->spai = new Spai();
  Spai *S = pc->spai;
  S->n = n;
  S->k = k;
  int st = ABX_OK;
  const auto t0 = std::chrono::steady_clock::now();
  DevBuf<float> feats, y;
  DevBuf<double> d2;
  PhaseEvents ev(p->ctx->stream);
  if ((st = S->cols.reserve((size_t)n * k + 1)) || (st = S->vals.reserve((size_t)n * k + 1)) ||
      (st = feats.reserve((size_t)n * k * p->dim + 1)) || (st = y.reserve((size_t)n * k + 1)) ||
      (st = d2.reserve((size_t)n * k + 1)) ||
      (n > 0 && ((ev.mark(0), st = knn_device(p, k, S->cols.ptr, d2.ptr)) ||
                 (ev.mark(1), st = spai_features_device(p, S->cols.ptr, k, eps, feats.ptr)) ||
                 // the model may live on another context (stream) of the same
                 // device: order its inference after the features and the
                 // weights' use after the inference
                 (ev.mark(2), st = stream_order(p->ctx->stream, mlp_context(mlp)->stream)) ||
                 (st = precision == ABX_PREC_FP64
                           ? mlp_infer_fp32(mlp, feats.ptr, n, y.ptr)
                           : mlp_infer_bf16(mlp, feats.ptr, n, y.ptr)) ||
                 (st = stream_order(mlp_context(mlp)->stream, p->ctx->stream))))) {
    delete pc->spai;
    delete pc;
    return st;
  }
  if (n > 0) ev.mark(3);
  if (n > 0) {
    k_f2d_masked<<<ceil_div((size_t)n * k, 256), 256, 0, p->ctx->stream>>>(y.ptr, S->cols.ptr,
                                                                          (size_t)n * k,
                                                                          S->vals.ptr);
    // rows next to a close neighbour: exact FP64 local-inverse rows
    DevBuf<int32_t> list;
    DevBuf<int> cnt;
    int nexact = 0;
    cudaError_t e = cudaSuccess;
    if (exact_phi < 1.0 && k >= 2) {
      if ((st = list.reserve((size_t)n)) || (st = cnt.reserve(1))) {
        delete pc->spai;
        delete pc;
        return st;
      }
      cudaMemsetAsync(cnt.ptr, 0, sizeof(int), p->ctx->stream);
      k_flag_close<<<ceil_div((size_t)n, 256), 256, 0, p->ctx->stream>>>(
          d2.ptr, n, k, op->k.kind, op->k.p[0], exact_phi, list.ptr, cnt.ptr);
      e = cudaMemcpyAsync(&nexact, cnt.ptr, sizeof(int), cudaMemcpyDeviceToHost, p->ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(p->ctx->stream);
      if (e == cudaSuccess && nexact > 0 &&
          (st = spai_exact_rows(op, k, S->cols.ptr, S->vals.ptr, 1, list.ptr, nexact, true))) {
        delete pc->spai;
        delete pc;
        return st;
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->ctx->stream);
    if (e != cudaSuccess) {
      delete pc->spai;
      delete pc;
      set_error("learned preconditioner: %s", cudaGetErrorString(e));
      return ABX_ERR_CUDA;
    }
    pc->exact_rows = nexact;
    ev.mark(4);
    ev.elapsed(pc->phase_s);
  }
  pc->setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ctx_retain(pc->ctx);
  *out = pc;
  return ABX_OK;
}

extern "C" int abx_precond_get_spai(abx_precond *pc, int32_t *cols, double *vals) {
  ABX_REQUIRE(pc && pc->kind == 2 && pc->spai, ABX_ERR_INVALID, "not a sparse approximate inverse");
  ABX_TRY(ctx_activate(pc->ctx));
  const size_t nk = (size_t)pc->spai->n * pc->spai->k;
  if (cols) ABX_CHECK_CUDA(cudaMemcpy(cols, pc->spai->cols.ptr, nk * 4, cudaMemcpyDefault));
  if (vals) ABX_CHECK_CUDA(cudaMemcpy(vals, pc->spai->vals.ptr, nk * 8, cudaMemcpyDefault));
  return ABX_OK;
}

extern "C" int abx_spai_local_inverse_rows(abx_operator *op, int k, int32_t *cols, double *vals) {
  ABX_REQUIRE(op && cols && vals, ABX_ERR_INVALID, "null argument");
  ABX_TRY(ctx_activate(op->rows->ctx));
  const int64_t n = op->rows->n;
  HostStage sc, sv;
  void *dc, *dv;
  ABX_TRY(sc.out(op->rows->ctx, cols, (size_t)n * k * 4, &dc));
  ABX_TRY(sv.out(op->rows->ctx, vals, (size_t)n * k * 8, &dv));
  ABX_TRY(spai_exact_rows(op, k, (int32_t *)dc, (double *)dv, 1));
  ABX_TRY(sc.finish(op->rows->ctx, cols, (size_t)n * k * 4));
  ABX_TRY(sv.finish(op->rows->ctx, vals, (size_t)n * k * 8));
  return ABX_OK;
}
