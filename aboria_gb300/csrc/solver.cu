// Preconditioners and the Krylov solver: restricted additive Schwarz on
// octree leaves, and restarted flexible GMRES with FP64 orthogonalisation and
// iterative refinement against an FP64 operator.
//
// Reference: SchwartzPreconditioner (src/Preconditioners.h:1121-1537):
//  * analyze_impl_block (:1170-1316): one domain per non-empty leaf; its
//    "indices" are the leaf's particles, its "buffer" the particles of every
//    bucket within L-infinity distance 1 of the leaf centre after scaling by
//    1/(half-width + 1e5*eps), i.e. all touching leaves.
//  * factorize (:1403-1467): dense block over indices ++ buffer assembled with
//    mat.coeff(i,j) (strict |dx|^2 < r^2, periodic-corrected dx:
//    src/detail/Kernels.h:336-368, src/Particles.h:480-496), then factorised.
//  * _solve_impl (:1477-1522): x = b; per domain gather b over indices ++
//    buffer, solve, scatter only the indices entries (restricted AS).
// The reference's Krylov solvers are Eigen's (GMRES at
// tests/rbf_interpolation.h:360-370); Eigen is third party and not vendored,
// so the GMRES here is this library's own: restarted, right-preconditioned
// flexible GMRES (FGMRES) with classical Gram-Schmidt and one
// re-orthogonalisation (CGS2), Givens rotations in FP64, and the true
// residual b - A x recomputed with an FP64 operator at every restart.
//
// GB300 layout: every domain's dense block lives in one FP64 arena
// (column-major, sum of n_d^2 doubles); factorisation is one CTA per domain,
// right-looking blocked LU with partial pivoting (panel width 32, trailing
// update tiled through shared memory); the apply is one CTA per domain
// (gather, pivots, two triangular solves with the columns streamed).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "handles.cuh"

namespace abx {

struct Schwarz {
  abx_operator *op = nullptr;
  int64_t n = 0;
  int ndom = 0;
  int max_size = 0;
  int precision = ABX_PREC_FP64;
  // per domain: offset into idx list, size, own count, matrix offset
  DevBuf<int> dom_off, dom_size, dom_own;
  DevBuf<int64_t> dom_mat;
  DevBuf<int> idx;       // concatenated particle indices (storage order): own first
  DevBuf<double> mat;    // LU factors, column-major per domain
  DevBuf<float> mat32;   // FP32 factors (mixed precision variant)
  DevBuf<int> piv;       // pivots per domain (offset dom_off)
  DevBuf<int> info;      // per-domain status (0 ok, k+1: zero pivot at k)
  double setup_s = 0.0;
  int64_t mat_elems = 0;
};

}  // namespace abx

namespace abx {
int spai_apply_device(abx_precond *pc, const double *b, double *x);  // spai.cu
void spai_free(abx_precond *pc);

namespace {

constexpr int TPB = 256;

// ------------------------------------------------------------ assembly ---
struct AsmParams {
  int dim, kind;
  double p0, r2;
  double L[3];
  int periodic[3];
  const double *pos;  // SoA storage order
  int64_t n;
  const int *dom_off, *dom_size;
  const int64_t *dom_mat;
  const int *idx;
  double *mat;
};

template <int KIND> __device__ __forceinline__ double coeff_val(double d2, double p0) {
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
  return 0.0;
}

// sparse_kernel::operator() (src/detail/Kernels.h:336-368): dx corrected for
// periodicity (src/Particles.h:480-496), value if |dx|^2 < r^2 (strict).
// One thread per matrix entry; column-major block per domain.
template <int KIND> __global__ void k_assemble(AsmParams P, int d0) {
  const int d = d0 + blockIdx.y;
  const int n = P.dom_size[d];
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * n) return;
  const int col = (int)(e / n), row = (int)(e % n);
  const int pi = P.idx[P.dom_off[d] + row], pj = P.idx[P.dom_off[d] + col];
  double d2 = 0.0;
  for (int k = 0; k < P.dim; ++k) {
    double dx = __dsub_rn(P.pos[(int64_t)k * P.n + pj], P.pos[(int64_t)k * P.n + pi]);
    if (P.periodic[k]) {
      const double w = P.L[k];
      while (dx > w / 2) dx -= w;
      while (dx <= -w / 2) dx += w;
    }
    d2 = __dadd_rn(d2, __dmul_rn(dx, dx));
  }
  P.mat[P.dom_mat[d] + e] = (d2 < P.r2) ? coeff_val<KIND>(d2, P.p0) : 0.0;
}

// -------------------------------------------------------- batched LU ---
constexpr int PW = 32;    // panel width
constexpr int LU_T = 256; // threads per CTA
constexpr int TB = 64;    // trailing-update tile

__device__ __forceinline__ double &M(double *A, int n, int r, int c) {
  return A[(int64_t)c * n + r];
}

// One CTA factorises one domain block in place: P A = L U (unit L).
__global__ void __launch_bounds__(LU_T) k_lu_fp64(double *__restrict__ mat,
                                                  const int64_t *__restrict__ dom_mat,
                                                  const int *__restrict__ dom_size,
                                                  const int *__restrict__ dom_off,
                                                  int *__restrict__ piv, int *__restrict__ info) {
  const int d = blockIdx.x;
  const int n = dom_size[d];
  double *A = mat + dom_mat[d];
  int *pv = piv + dom_off[d];
  __shared__ double red_v[LU_T / 32];
  __shared__ int red_i[LU_T / 32];
  __shared__ int s_piv;
  __shared__ double sL[TB][PW + 1];
  __shared__ double sU[PW][TB + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int status = 0;
  for (int k0 = 0; k0 < n; k0 += PW) {
    const int kw = min(PW, n - k0);
    // ---- panel factorisation, column by column
    for (int c = k0; c < k0 + kw; ++c) {
      // pivot search over rows c..n-1 of column c
      double best = -1.0;
      int bi = c;
      for (int r = c + tid; r < n; r += LU_T) {
        const double v = fabs(M(A, n, r, c));
        if (v > best) { best = v; bi = r; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
      }
      if (lane == 0) { red_v[warp] = best; red_i[warp] = bi; }
      __syncthreads();
      if (tid == 0) {
        double bv = red_v[0];
        int bj = red_i[0];
        for (int w = 1; w < LU_T / 32; ++w)
          if (red_v[w] > bv || (red_v[w] == bv && red_i[w] < bj)) { bv = red_v[w]; bj = red_i[w]; }
        s_piv = bj;
        pv[c] = bj;
        if (bv == 0.0 && status == 0) status = c + 1;
      }
      __syncthreads();
      const int p = s_piv;
      if (p != c) {  // swap whole rows c and p (LAPACK getrf convention)
        for (int j = tid; j < n; j += LU_T) {
          const double t = M(A, n, c, j);
          M(A, n, c, j) = M(A, n, p, j);
          M(A, n, p, j) = t;
        }
      }
      __syncthreads();
      const double dpiv = M(A, n, c, c);
      const double inv = dpiv != 0.0 ? 1.0 / dpiv : 0.0;
      for (int r = c + 1 + tid; r < n; r += LU_T) M(A, n, r, c) *= inv;
      __syncthreads();
      // rank-1 update of the rest of the panel
      for (int cc = c + 1; cc < k0 + kw; ++cc) {
        const double u = M(A, n, c, cc);
        for (int r = c + 1 + tid; r < n; r += LU_T) M(A, n, r, cc) -= M(A, n, r, c) * u;
      }
      __syncthreads();
    }
    const int k1 = k0 + kw;
    if (k1 >= n) break;
    // ---- U12 = L11^{-1} A12 (unit lower triangular solve), columns in parallel
    for (int j = k1 + tid; j < n; j += LU_T) {
      for (int c = k0; c < k1; ++c) {
        const double u = M(A, n, c, j);
        for (int r = c + 1; r < k1; ++r) M(A, n, r, j) -= M(A, n, r, c) * u;
      }
    }
    __syncthreads();
    // ---- A22 -= L21 * U12, 64x64 tiles, each thread a 4x4 micro-tile
    for (int ti = k1; ti < n; ti += TB) {
      for (int tj = k1; tj < n; tj += TB) {
        // stage L21 tile (rows ti.., cols k0..k1) and U12 tile (rows k0..k1, cols tj..)
        for (int e = tid; e < TB * PW; e += LU_T) {
          const int r = e % TB, c = e / TB;
          sL[r][c] = (ti + r < n && c < kw) ? M(A, n, ti + r, k0 + c) : 0.0;
        }
        for (int e = tid; e < PW * TB; e += LU_T) {
          const int r = e % PW, c = e / PW;
          sU[r][c] = (tj + c < n && r < kw) ? M(A, n, k0 + r, tj + c) : 0.0;
        }
        __syncthreads();
        const int tr = (tid % 16) * 4, tc = (tid / 16) * 4;
        double acc[4][4] = {};
        for (int c = 0; c < kw; ++c) {
          double a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) a[i] = sL[tr + i][c];
#pragma unroll
          for (int j = 0; j < 4; ++j) b[j] = sU[c][tc + j];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int cj = tj + tc + j;
          if (cj >= n) continue;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int ri = ti + tr + i;
            if (ri < n) M(A, n, ri, cj) -= acc[i][j];
          }
        }
        __syncthreads();
      }
    }
  }
  if (tid == 0) info[d] = status;
}

__global__ void k_to_f32(const double *__restrict__ a, int64_t n, float *__restrict__ b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// ----------------------------------------------------------- RAS apply ---
// x = b outside every domain's own set; for each domain: y = b[idx]; apply
// the row swaps; solve L (unit) then U; x[own] = y[own].  The block's columns
// are streamed: forward step j subtracts y_j * L[j+1:, j] from the rest.
template <class T>
__global__ void __launch_bounds__(LU_T) k_ras_apply(const T *__restrict__ mat,
                                                    const int64_t *__restrict__ dom_mat,
                                                    const int *__restrict__ dom_size,
                                                    const int *__restrict__ dom_off,
                                                    const int *__restrict__ dom_own,
                                                    const int *__restrict__ idx,
                                                    const int *__restrict__ piv,
                                                    const double *__restrict__ b,
                                                    double *__restrict__ x) {
  extern __shared__ double y[];
  const int d = blockIdx.x;
  const int n = dom_size[d];
  const T *A = mat + dom_mat[d];
  const int *id = idx + dom_off[d];
  const int *pv = piv + dom_off[d];
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += LU_T) y[i] = b[id[i]];
  __syncthreads();
  if (tid == 0)
    for (int c = 0; c < n; ++c) {
      const int p = pv[c];
      if (p != c) { const double t = y[c]; y[c] = y[p]; y[p] = t; }
    }
  __syncthreads();
  for (int c = 0; c < n; ++c) {  // L y = y
    const double yc = y[c];
    for (int r = c + 1 + tid; r < n; r += LU_T) y[r] -= (double)A[(int64_t)c * n + r] * yc;
    __syncthreads();
  }
  for (int c = n - 1; c >= 0; --c) {  // U y = y
    if (tid == 0) y[c] = y[c] / (double)A[(int64_t)c * n + c];
    __syncthreads();
    const double yc = y[c];
    for (int r = tid; r < c; r += LU_T) y[r] -= (double)A[(int64_t)c * n + r] * yc;
    __syncthreads();
  }
  const int own = dom_own[d];
  for (int i = tid; i < own; i += LU_T) x[id[i]] = y[i];
}

// -------------------------------------------------------------- GMRES ---
__global__ void k_copy(const double *__restrict__ a, int64_t n, double *__restrict__ b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

// y = a x (y is not read: it may hold uninitialised memory)
__global__ void k_scale(int64_t n, double a, const double *__restrict__ x,
                        double *__restrict__ y) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = a * x[i];
}

__global__ void k_sub(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                      double *__restrict__ out) {  // out = a - b
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}

// h[k] += sum_i V[k][i] * w[i] for k < m (one block row of partial sums per
// CTA, reduced on the host side of the call by k_reduce_rows).
constexpr int DOT_CTAS = 304;
__global__ void k_multidot(const double *__restrict__ V, int64_t ldv, int m,
                           const double *__restrict__ w, int64_t n, double *__restrict__ part) {
  // part[k * DOT_CTAS + blockIdx.x]
  __shared__ double red[TPB / 32];
  for (int k = 0; k < m; ++k) {
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * TPB + threadIdx.x; i < n; i += (int64_t)gridDim.x * TPB)
      s = fma(V[k * ldv + i], w[i], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int i = 0; i < TPB / 32; ++i) t += red[i];
      part[(int64_t)k * gridDim.x + blockIdx.x] = t;
    }
    __syncthreads();
  }
}

__global__ void k_reduce_rows(const double *__restrict__ part, int m, int ncta,
                              double *__restrict__ h) {
  const int k = blockIdx.x;
  if (k >= m) return;
  double s = 0.0;
  for (int i = threadIdx.x; i < ncta; i += blockDim.x) s += part[(int64_t)k * ncta + i];
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) t += red[i];
    h[k] = t;
  }
}

// w -= V[0:m]^T h
__global__ void k_sub_vh(double *__restrict__ w, const double *__restrict__ V, int64_t ldv, int m,
                         const double *__restrict__ h, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = w[i];
  for (int k = 0; k < m; ++k) s -= V[k * ldv + i] * h[k];
  w[i] = s;
}

// x += Z[0:m]^T y
__global__ void k_add_zy(double *__restrict__ x, const double *__restrict__ Z, int64_t ldz, int m,
                         const double *__restrict__ y, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = x[i];
  for (int k = 0; k < m; ++k) s += Z[k * ldz + i] * y[k];
  x[i] = s;
}

}  // namespace

// ------------------------------------------------------------- host side ---
namespace {

// Leaves whose boxes touch `box` (grown by `grow` per side): tree descent.
void touching_leaves(const abx_particles *p, const double *lo, const double *hi, double grow,
                     std::vector<int> &out) {
  const OctTree &T = p->tree;
  std::vector<int> stack(1, 0);
  while (!stack.empty()) {
    const int nd = stack.back();
    stack.pop_back();
    if (T.kind[nd] == 0) continue;
    double blo[3], bhi[3];
    T.box(p->grid, nd, blo, bhi);
    bool overlap = true;
    for (int d = 0; d < p->dim; ++d)
      if (bhi[d] < lo[d] - grow || blo[d] > hi[d] + grow) overlap = false;
    if (!overlap) continue;
    if (T.kind[nd] == 1) {
      out.push_back(nd);
    } else {
      const int nc = 1 << p->dim;
      for (int c = nc - 1; c >= 0; --c) stack.push_back(T.first_child[nd] + c);
    }
  }
}

int launch_assemble(abx_context *ctx, const Schwarz &S, const abx_particles *p, const abx_kernel &k,
                    double radius, const std::vector<int> &sizes) {
  AsmParams P{};
  P.dim = p->dim;
  P.kind = k.kind;
  P.p0 = k.p[0];
  P.r2 = radius * radius;  // std::pow(m_fradius(a), 2)
  for (int d = 0; d < 3; ++d) {
    P.L[d] = p->grid.hi[d] - p->grid.lo[d];
    P.periodic[d] = d < p->dim ? p->grid.periodic[d] : 0;
  }
  P.pos = p->pos.ptr;
  P.n = p->n;
  P.dom_off = S.dom_off.ptr;
  P.dom_size = S.dom_size.ptr;
  P.dom_mat = S.dom_mat.ptr;
  P.idx = S.idx.ptr;
  P.mat = S.mat.ptr;
  // one launch per group of domains with similar size bound
  for (int d0 = 0; d0 < S.ndom; d0 += 1024) {
    const int nd = std::min(1024, S.ndom - d0);
    int mx = 0;
    for (int d = d0; d < d0 + nd; ++d) mx = std::max(mx, sizes[d]);
    dim3 grid(ceil_div((size_t)mx * mx, TPB), nd);
    switch (k.kind) {
    case ABX_K_CONST: k_assemble<ABX_K_CONST><<<grid, TPB, 0, ctx->stream>>>(P, d0); break;
    case ABX_K_GAUSSIAN: k_assemble<ABX_K_GAUSSIAN><<<grid, TPB, 0, ctx->stream>>>(P, d0); break;
    case ABX_K_WENDLAND_C2: k_assemble<ABX_K_WENDLAND_C2><<<grid, TPB, 0, ctx->stream>>>(P, d0); break;
    case ABX_K_COMPACT_GAUSSIAN:
      k_assemble<ABX_K_COMPACT_GAUSSIAN><<<grid, TPB, 0, ctx->stream>>>(P, d0);
      break;
    case ABX_K_LAPLACE: k_assemble<ABX_K_LAPLACE><<<grid, TPB, 0, ctx->stream>>>(P, d0); break;
    case ABX_K_MULTIQUADRIC: k_assemble<ABX_K_MULTIQUADRIC><<<grid, TPB, 0, ctx->stream>>>(P, d0); break;
    default:
      set_error("Schwarz: kernel kind %d not supported", k.kind);
      return ABX_ERR_INVALID;
    }
    ABX_CHECK_CUDA(cudaGetLastError());
  }
  return ABX_OK;
}

}  // namespace

int schwarz_build(abx_operator *op, int precision, Schwarz *&out) {
  abx_particles *p = op->rows;
  abx_context *ctx = p->ctx;
  ABX_REQUIRE(op->kind == 0, ABX_ERR_INVALID, "Schwarz preconditioner needs a sparse operator");
  ABX_REQUIRE(op->rows == op->cols, ABX_ERR_INVALID,
              "Schwartz preconditioner restricted to identical row and col particle sets");
  ABX_REQUIRE(p->searchable && p->search_kind == 1, ABX_ERR_STATE,
              "Schwarz domains are octree leaves: call abx_particles_init_octree first");
  ABX_REQUIRE(op->k.kind != ABX_K_SCALAR_SUM, ABX_ERR_INVALID,
              "Schwarz: ABX_K_SCALAR_SUM not supported");
  const auto t0 = std::chrono::steady_clock::now();
  Schwarz *S = new Schwarz();
  S->op = op;
  S->n = p->n;
  S->precision = precision;
  const OctTree &T = p->tree;
  const double eps_buf = 1e5 * 2.220446049250313e-16;  // m_neighbourhood_buffer
  std::vector<int> off, size, own, idx;
  std::vector<int64_t> moff;
  int64_t mtot = 0;
  std::vector<int> touch;
  for (int leaf : T.leaves) {
    if (T.end[leaf] <= T.begin[leaf]) continue;
    double lo[3], hi[3];
    T.box(p->grid, leaf, lo, hi);
    touch.clear();
    touching_leaves(p, lo, hi, eps_buf, touch);
    off.push_back((int)idx.size());
    const int own_n = T.end[leaf] - T.begin[leaf];
    for (int i = T.begin[leaf]; i < T.end[leaf]; ++i) idx.push_back(i);
    for (int nb : touch)
      if (nb != leaf)
        for (int i = T.begin[nb]; i < T.end[nb]; ++i) idx.push_back(i);
    const int sz = (int)idx.size() - off.back();
    size.push_back(sz);
    own.push_back(own_n);
    moff.push_back(mtot);
    mtot += (int64_t)sz * sz;
    S->max_size = std::max(S->max_size, sz);
  }
  S->ndom = (int)size.size();
  S->mat_elems = mtot;
  int st = ABX_OK;
  auto fail = [&](int s) {
    delete S;
    return s;
  };
  if ((st = S->dom_off.reserve(S->ndom + 1)) || (st = S->dom_size.reserve(S->ndom + 1)) ||
      (st = S->dom_own.reserve(S->ndom + 1)) || (st = S->dom_mat.reserve(S->ndom + 1)) ||
      (st = S->idx.reserve(idx.size() + 1)) || (st = S->piv.reserve(idx.size() + 1)) ||
      (st = S->info.reserve(S->ndom + 1)) || (st = S->mat.reserve(mtot + 1)))
    return fail(st);
  cudaStream_t s = ctx->stream;
  if (S->ndom > 0) {
    cudaMemcpyAsync(S->dom_off.ptr, off.data(), off.size() * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(S->dom_size.ptr, size.data(), size.size() * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(S->dom_own.ptr, own.data(), own.size() * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(S->dom_mat.ptr, moff.data(), moff.size() * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(S->idx.ptr, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, s);
    if ((st = launch_assemble(ctx, *S, p, op->k, op->radius, size))) return fail(st);
    k_lu_fp64<<<S->ndom, LU_T, 0, s>>>(S->mat.ptr, S->dom_mat.ptr, S->dom_size.ptr,
                                        S->dom_off.ptr, S->piv.ptr, S->info.ptr);
    if (cudaGetLastError() != cudaSuccess) {
      set_error("LU launch failed");
      return fail(ABX_ERR_CUDA);
    }
    if (precision == ABX_PREC_MIXED) {
      if ((st = S->mat32.reserve(mtot + 1))) return fail(st);
      k_to_f32<<<ceil_div(mtot, TPB), TPB, 0, s>>>(S->mat.ptr, mtot, S->mat32.ptr);
      S->mat.release();
    }
    std::vector<int> info(S->ndom);
    cudaMemcpyAsync(info.data(), S->info.ptr, S->ndom * 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      set_error("Schwarz factorisation: %s", cudaGetErrorString(e));
      return fail(ABX_ERR_CUDA);
    }
    for (int d = 0; d < S->ndom; ++d)
      if (info[d] != 0) {
        set_error("Schwarz: domain %d block is singular (zero pivot at %d)", d, info[d] - 1);
        return fail(ABX_ERR_NUMERIC);
      }
  }
  S->setup_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  out = S;
  return ABX_OK;
}

int schwarz_apply_device(Schwarz *S, abx_context *ctx, const double *b, double *x) {
  cudaStream_t s = ctx->stream;
  if (S->n == 0) return ABX_OK;
  k_copy<<<ceil_div(S->n, TPB), TPB, 0, s>>>(b, S->n, x);
  const size_t smem = (size_t)S->max_size * sizeof(double);
  if (smem > 48 * 1024) {
    if (S->precision == ABX_PREC_MIXED)
      ABX_CHECK_CUDA(cudaFuncSetAttribute(k_ras_apply<float>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    else
      ABX_CHECK_CUDA(cudaFuncSetAttribute(k_ras_apply<double>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  ABX_REQUIRE(smem <= 227 * 1024, ABX_ERR_CAPACITY, "Schwarz domain of %d particles too large",
              S->max_size);
  if (S->ndom > 0) {
    if (S->precision == ABX_PREC_MIXED)
      k_ras_apply<float><<<S->ndom, LU_T, smem, s>>>(S->mat32.ptr, S->dom_mat.ptr, S->dom_size.ptr,
                                                     S->dom_off.ptr, S->dom_own.ptr, S->idx.ptr,
                                                     S->piv.ptr, b, x);
    else
      k_ras_apply<double><<<S->ndom, LU_T, smem, s>>>(S->mat.ptr, S->dom_mat.ptr, S->dom_size.ptr,
                                                      S->dom_off.ptr, S->dom_own.ptr, S->idx.ptr,
                                                      S->piv.ptr, b, x);
    ABX_CHECK_CUDA(cudaGetLastError());
  }
  return ABX_OK;
}

int precond_apply_device(abx_precond *pc, const double *b, double *x) {
  if (!pc) return ABX_OK;
  if (pc->kind == 1) return schwarz_apply_device(pc->schwarz, pc->ctx, b, x);
  if (pc->kind == 2) return spai_apply_device(pc, b, x);
  set_error("unknown preconditioner kind %d", pc->kind);
  return ABX_ERR_INVALID;
}

int sparse_or_dense_matvec(abx_operator *op, const double *b, double *c) {
  if (op->kind == 0) return sparse_matvec_device(op, b, c);
  if (op->kind == 1) return dense_matvec_device(op, b, c);
  return fmm_matvec_device(op, b, c);
}

// ------------------------------------------------------------- FGMRES ---
struct GmresWork {
  DevBuf<double> V, Z, w, r, part, h, tmp;
};

int gmres_solve(abx_operator *A, abx_operator *Acheck, abx_precond *M, const double *b, double *x,
                int restart, int max_iters, double tol, int *iters_out, double *resid_out,
                int *restarts_out) {
  abx_context *ctx = A->rows->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t n = A->rows->n;
  ABX_REQUIRE(A->rows->n == A->cols->n, ABX_ERR_INVALID, "GMRES needs a square operator");
  ABX_REQUIRE(restart >= 1 && restart <= 1000, ABX_ERR_INVALID, "restart out of range");
  if (!Acheck) Acheck = A;
  GmresWork W;
  const int m = restart;
  ABX_TRY(W.V.reserve((size_t)(m + 1) * n + 1));
  ABX_TRY(W.Z.reserve((size_t)m * n + 1));
  ABX_TRY(W.w.reserve(n + 1));
  ABX_TRY(W.r.reserve(n + 1));
  ABX_TRY(W.part.reserve((size_t)(m + 1) * DOT_CTAS + 1));
  ABX_TRY(W.h.reserve(m + 2));
  ABX_TRY(W.tmp.reserve(n + 1));
  const unsigned nb = ceil_div(n, TPB);
  auto dot_many = [&](const double *V, int k, const double *v, double *hdev, double *hhost) -> int {
    k_multidot<<<DOT_CTAS, TPB, 0, s>>>(V, n, k, v, n, W.part.ptr);
    k_reduce_rows<<<k, 256, 0, s>>>(W.part.ptr, k, DOT_CTAS, hdev);
    ABX_CHECK_CUDA(cudaGetLastError());
    if (hhost) {
      ABX_CHECK_CUDA(cudaMemcpyAsync(hhost, hdev, k * sizeof(double), cudaMemcpyDeviceToHost, s));
      ABX_CHECK_CUDA(cudaStreamSynchronize(s));
    }
    return ABX_OK;
  };
  auto norm = [&](const double *v, double &out) -> int {
    double h;
    ABX_TRY(dot_many(v, 1, v, W.h.ptr, &h));
    out = std::sqrt(std::max(h, 0.0));
    return ABX_OK;
  };
  double bnorm;
  ABX_TRY(norm(b, bnorm));
  if (bnorm == 0.0) {
    ABX_CHECK_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    *iters_out = 0;
    *resid_out = 0.0;
    return ABX_OK;
  }
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hcol(m + 2), h2(m + 2), y(m);
  int total = 0, restarts = 0;
  double rel = 1.0;
  // refinement (a less accurate Krylov operator than A_check): the inner
  // cycle's target relative to the current true residual.  It starts at 1e-5;
  // after each cycle it follows half the contraction that cycle achieved on
  // the checked residual -- iterating the inner system far below what the
  // operator difference lets the outer residual gain is wasted work.
  const bool refining = Acheck != A && Acheck->precision != A->precision;
  double inner_ratio = 1e-5, prev_beta = -1.0;
  for (;;) {
    // true residual with the checking operator
    ABX_TRY(sparse_or_dense_matvec(Acheck, x, W.tmp.ptr));
    k_sub<<<nb, TPB, 0, s>>>(n, b, W.tmp.ptr, W.r.ptr);
    double beta;
    ABX_TRY(norm(W.r.ptr, beta));
    rel = beta / bnorm;
    if (!(rel == rel)) {
      set_error("GMRES: non-finite residual");
      return ABX_ERR_NUMERIC;
    }
    if (rel <= tol || total >= max_iters) break;
    if (refining && prev_beta > 0.0)
      inner_ratio = std::min(0.5, std::max(1e-5, 0.5 * beta / prev_beta));
    prev_beta = beta;
    k_scale<<<nb, TPB, 0, s>>>(n, 1.0 / beta, W.r.ptr, W.V.ptr);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    // inner tolerance: when the Krylov operator is less accurate than the
    // checking operator (mixed precision), each cycle only reduces the
    // residual by inner_ratio and the restart (a refinement step against
    // A_check) does the rest.
    const double target = std::max(tol * bnorm, refining ? inner_ratio * beta : 0.0);
    for (; j < m && total < max_iters; ++j, ++total) {
      double *vj = W.V.ptr + (size_t)j * n;
      double *zj = W.Z.ptr + (size_t)j * n;
      if (M) {
        ABX_TRY(precond_apply_device(M, vj, zj));
      } else {
        k_copy<<<nb, TPB, 0, s>>>(vj, n, zj);
      }
      ABX_TRY(sparse_or_dense_matvec(A, zj, W.w.ptr));
      // CGS2: two passes of classical Gram-Schmidt
      std::fill(hcol.begin(), hcol.end(), 0.0);
      for (int pass = 0; pass < 2; ++pass) {
        ABX_TRY(dot_many(W.V.ptr, j + 1, W.w.ptr, W.h.ptr, h2.data()));
        k_sub_vh<<<nb, TPB, 0, s>>>(W.w.ptr, W.V.ptr, n, j + 1, W.h.ptr, n);
        for (int i = 0; i <= j; ++i) hcol[i] += h2[i];
      }
      double hn;
      ABX_TRY(norm(W.w.ptr, hn));
      hcol[j + 1] = hn;
      if (hn > 0.0) k_scale<<<nb, TPB, 0, s>>>(n, 1.0 / hn, W.w.ptr, W.V.ptr + (size_t)(j + 1) * n);
      // apply previous rotations, then a new one
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
        hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
        hcol[i] = t;
      }
      const double den = std::hypot(hcol[j], hcol[j + 1]);
      cs[j] = den > 0 ? hcol[j] / den : 1.0;
      sn[j] = den > 0 ? hcol[j + 1] / den : 0.0;
      hcol[j] = den;
      hcol[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hcol[i];
      if (std::fabs(g[j + 1]) <= target || hn == 0.0) {
        ++j;
        ++total;
        break;
      }
    }
    // back substitution for y, then x += Z y
    for (int i = j - 1; i >= 0; --i) {
      double t = g[i];
      for (int k = i + 1; k < j; ++k) t -= H[(size_t)i * m + k] * y[k];
      y[i] = H[(size_t)i * m + i] != 0.0 ? t / H[(size_t)i * m + i] : 0.0;
    }
    if (j > 0) {
      ABX_CHECK_CUDA(cudaMemcpyAsync(W.h.ptr, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, s));
      k_add_zy<<<nb, TPB, 0, s>>>(x, W.Z.ptr, n, j, W.h.ptr, n);
      ABX_CHECK_CUDA(cudaGetLastError());
    }
    ++restarts;
  }
  ABX_CHECK_CUDA(cudaStreamSynchronize(s));
  *iters_out = total;
  *resid_out = rel;
  if (restarts_out) *restarts_out = restarts;
  return ABX_OK;
}

}  // namespace abx

using namespace abx;

extern "C" {

int abx_precond_create_schwarz(abx_operator *op, int precision, abx_precond **out) {
  ABX_REQUIRE(op && out, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(precision == ABX_PREC_FP64 || precision == ABX_PREC_MIXED, ABX_ERR_INVALID,
              "unknown precision %d", precision);
  ABX_TRY(ctx_activate(op->rows->ctx));
  if (!op->pairs) ABX_TRY(pair_layout_build(op));
  Schwarz *S = nullptr;
  ABX_TRY(schwarz_build(op, precision, S));
  abx_precond *pc = new abx_precond();
  pc->kind = 1;
  pc->schwarz = S;
  pc->ctx = op->rows->ctx;
  pc->n = op->rows->n;
  ctx_retain(pc->ctx);
  *out = pc;
  return ABX_OK;
}

int abx_precond_destroy(abx_precond *pc) {
  if (!pc) return ABX_OK;
  abx_context *ctx = pc->ctx;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (pc->schwarz) delete pc->schwarz;
  if (pc->spai) spai_free(pc);
  delete pc;
  ctx_release(ctx);
  return ABX_OK;
}

int abx_precond_apply(abx_precond *pc, const double *b, double *x) {
  ABX_REQUIRE(pc, ABX_ERR_INVALID, "null preconditioner");
  ABX_TRY(ctx_activate(pc->ctx));
  const void *bd;
  void *xd;
  ABX_TRY(pc->stage_b.in(pc->ctx, b, pc->n * sizeof(double), &bd));
  ABX_TRY(pc->stage_x.out(pc->ctx, x, pc->n * sizeof(double), &xd));
  ABX_TRY(precond_apply_device(pc, (const double *)bd, (double *)xd));
  ABX_TRY(pc->stage_x.finish(pc->ctx, x, pc->n * sizeof(double)));
  return ABX_OK;
}

int abx_precond_setup_phases(abx_precond *pc, double *knn_s, double *features_s, double *infer_s,
                             double *exact_s) {
  ABX_REQUIRE(pc, ABX_ERR_INVALID, "null preconditioner");
  double *out[4] = {knn_s, features_s, infer_s, exact_s};
  for (int i = 0; i < 4; ++i)
    if (out[i]) *out[i] = pc->phase_s[i];
  return ABX_OK;
}

int abx_precond_stats(abx_precond *pc, int64_t *ndomains, int64_t *max_size, int64_t *elements,
                      double *setup_seconds) {
  ABX_REQUIRE(pc, ABX_ERR_INVALID, "null preconditioner");
  if (pc->kind == 1) {
    if (ndomains) *ndomains = pc->schwarz->ndom;
    if (max_size) *max_size = pc->schwarz->max_size;
    if (elements) *elements = pc->schwarz->mat_elems;
    if (setup_seconds) *setup_seconds = pc->schwarz->setup_s;
  } else {
    // approximate inverse: ndomains = rows solved exactly (learned: the rows
    // next to a close neighbour); no domains or stored blocks
    if (ndomains) *ndomains = pc->exact_rows;
    if (max_size) *max_size = 0;
    if (elements) *elements = 0;
    if (setup_seconds) *setup_seconds = pc->setup_s;
  }
  return ABX_OK;
}

int abx_gmres_solve(abx_operator *A, abx_operator *A_check, abx_precond *M, const double *b,
                    double *x, int restart, int max_iters, double tol, int *iterations,
                    double *rel_residual) {
  ABX_REQUIRE(A && b && x && iterations && rel_residual, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(!A_check || (A_check->rows == A->rows && A_check->cols == A->cols), ABX_ERR_INVALID,
              "the checking operator must act on the same particle sets");
  abx_context *ctx = A->rows->ctx;
  ABX_TRY(ctx_activate(ctx));
  const int64_t n = A->rows->n;
  HostStage sb, sx;
  const void *bd;
  void *xd;
  ABX_TRY(sb.in(ctx, b, n * sizeof(double), &bd));
  // x is in/out: stage it in, solve, stage it back
  const void *x_in;
  ABX_TRY(sx.in(ctx, x, n * sizeof(double), &x_in));
  xd = const_cast<void *>(x_in);
  int restarts = 0;
  const int st = gmres_solve(A, A_check, M, (const double *)bd, (double *)xd, restart, max_iters,
                             tol, iterations, rel_residual, &restarts);
  if (st != ABX_OK) return st;
  if (xd != (void *)x) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(x, xd, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    ABX_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return ABX_OK;
}

}  // extern "C"

extern "C" int abx_gmres_solve_fallback(abx_operator *A, abx_operator *A_check,
                                        abx_precond *M_learned, abx_operator *A_fallback,
                                        const double *b, double *x, int restart,
                                        int learned_max_iters, int max_iters, double tol,
                                        int *iterations, double *rel_residual,
                                        int *used_fallback) {
  ABX_REQUIRE(A && b && x && iterations && rel_residual && used_fallback, ABX_ERR_INVALID,
              "null argument");
  abx_context *ctx = A->rows->ctx;
  ABX_TRY(ctx_activate(ctx));
  const int64_t n = A->rows->n;
  HostStage sb, sx;
  const void *bd, *x_in;
  ABX_TRY(sb.in(ctx, b, n * sizeof(double), &bd));
  ABX_TRY(sx.in(ctx, x, n * sizeof(double), &x_in));
  double *xd = (double *)const_cast<void *>(x_in);
  int it1 = 0, it2 = 0, restarts = 0;
  double res = 1.0;
  *used_fallback = 0;
  if (M_learned) {
    ABX_TRY(gmres_solve(A, A_check, M_learned, (const double *)bd, xd, restart,
                        std::min(learned_max_iters, max_iters), tol, &it1, &res, &restarts));
  }
  if (!(res <= tol) && A_fallback) {
    *used_fallback = 1;
    Schwarz *S = nullptr;
    if (!A_fallback->pairs) ABX_TRY(pair_layout_build(A_fallback));
    ABX_TRY(schwarz_build(A_fallback, ABX_PREC_FP64, S));
    abx_precond pc;
    pc.kind = 1;
    pc.schwarz = S;
    pc.ctx = ctx;
    pc.n = n;
    const int st = gmres_solve(A, A_check, &pc, (const double *)bd, xd, restart,
                               std::max(0, max_iters - it1), tol, &it2, &res, &restarts);
    pc.schwarz = nullptr;
    delete S;
    if (st != ABX_OK) return st;
  }
  *iterations = it1 + it2;
  *rel_residual = res;
  if ((void *)xd != (void *)x) {
    ABX_CHECK_CUDA(cudaMemcpyAsync(x, xd, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    ABX_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return ABX_OK;
}
