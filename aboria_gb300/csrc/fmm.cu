// Black-box Chebyshev FMM operator (create_fmm_operator, src/Operators.h:
// 401-407; KernelFMM src/Kernels.h:533-576).
//
// Reference algorithm (restated, not translated):
//  * expansions: BlackBoxExpansions (src/detail/FastMultipoleMethod.h:96-368)
//    with Chebyshev interpolation (src/detail/Chebyshev.h:84-153, 245-294):
//    R_j(x) = prod_d S_{m_d(j)}(x_d), nodes in lattice order (last dim fastest);
//  * traversal: FastMultipoleMethod::matrix_vector_multiply
//    (src/FastMultipoleMethod.h:111-548) with theta_condition
//    (src/detail/FastMultipoleMethod.h:1249-1279), P2P at target leaves over
//    the connected list (leaf or whole subtree).
//
// GB300 design: the traversal runs once per operator on the host and is
// flattened into per-level lists (M2L pairs, P2P leaf pairs, parent/child
// links); translation operators are precomputed instead of re-evaluating the
// kernel at node pairs on every call: one M2M/L2L matrix per child octant
// (the Chebyshev interpolation is scale invariant) and one M2L matrix per
// (level, box offset) -- M2L pairs at one level differ only by an integer box
// offset in [-3, 3]^D.  Each matvec is five passes of device kernels: P2M,
// M2M (bottom-up), M2L, L2L (top-down), then L2P+P2P per target leaf.
//
// M2L in the mixed-precision mode runs as a GEMM per (level, offset) on the
// tensor cores (3xTF32 split with FP32 accumulation, mma.sync m16n8k8):
//   G[:, targets] += K_o * W[:, sources]  (one CTA per 16-row x 64-target tile)
// and P2P in FP32; the FP64 mode keeps every pass in FP64.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <functional>
#include <map>
#include <vector>

#include "common.cuh"
#include "handles.cuh"

namespace abx {

constexpr int MAXN_TAB = 8;  // max Chebyshev order of the coefficient table

// Clenshaw coefficients of S_m: c[m][k] = (2/n) cos(k (2m+1) pi / (2n)).
struct ChebTab {
  double c[MAXN_TAB][MAXN_TAB];
};
struct ChebTab32 {  // the same in FP32 (mixed-precision P2M and L2P)
  float c[MAXN_TAB][MAXN_TAB];
};

struct FmmPlan {
  int D = 3, n = 3, ncheb = 27, nchild = 8;
  int nnodes = 0;
  int kind = 0;
  double p0 = 0.0;
  std::vector<int> mi;  // ncheb x D multi-indices
  // device
  DevBuf<double> W, G;            // nnodes x ncheb
  DevBuf<double> Tc;              // nchild x ncheb x ncheb (child->parent interpolation)
  DevBuf<float> Tc32;             // FP32 copy (mixed-precision L2L)
  DevBuf<double> TcT;             // transposed: TcT[o][j][i] = Tc[o][i][j] (M2M)
  DevBuf<float> Tc32T;            // FP32 copy of TcT (mixed-precision M2M)
  DevBuf<double> box;             // nnodes x 6 (lo[3], hi[3])
  DevBuf<int> leaf_ids;           // leaves (node ids)
  DevBuf<int> node_begin, node_end;
  // per level: nodes with children (M2M/L2L), (parent, child, octant) links
  std::vector<int> max_level;
  std::vector<std::vector<int>> level_links;  // host: flattened (parent, child, octant)
  DevBuf<int> links;                          // all levels, octant-major within a level
  DevBuf<int2> batches;                       // (first link, count <= NBL) of one octant
  std::vector<int> batch_off, batch_cnt;      // per level
  // M2L: pairs (target, source, matrix id), grouped by level
  DevBuf<int> m2l;
  int n_m2l = 0;
  DevBuf<double> Km;      // nmat x ncheb x ncheb
  DevBuf<float> Kmh, Kml; // split-TF32 hi/lo parts of the FP32 copy (mma.sync M2L, ncheb <= 64)
  DevBuf<float> Kp;       // the same packed as tcgen05 stage images (ncheb > 64, k_pack_tf32)
  DevBuf<float> W32l;     // lo part of W (the tcgen05 M2L reads W32 as the hi part)
  int nmat = 0;
  // M2L grouped by matrix (for the tensor-core GEMM): per matrix a list of
  // (target, source)
  DevBuf<int2> m2l_by_mat;
  std::vector<int> mat_off, mat_cnt;
  DevBuf<int> mat_off_d;
  // P2P: CSR over target leaves of source leaves
  DevBuf<int> p2p_rowptr, p2p_src;
  int nleaves = 0;
  double build_s = 0.0;
  double chebsetup_s = 0.0;
  // tcgen05 M2L: limit of each mbarrier wait, and the test-only fault
  // injection that withholds one operand-ready signal
  double wait_limit_s = 1.0;
  int drop_arrive = 0;
  DevBuf<float> W32, G32;
  ChebTab tab{};        // Clenshaw coefficients of the order
  ChebTab32 tab32{};    // the same in FP32 (mixed-precision P2M / L2P)
  DevBuf<float4> posf;  // mixed near field: FP32 position relative to the leaf centre
  DevBuf<float> b32;    // mixed near field: FP32 weights of the current matvec
  DevBuf<int> mi_d;                 // ncheb x 3 multi-indices
  DevBuf<int> tile_mat, tile_first; // tensor-core M2L tiles
  int ntiles = 0;
};

void fmm_plan_free(FmmPlan *P) { delete P; }

namespace {

constexpr double PI = 3.14159265358979323846;

// S_m(x), m = 0..n-1 (chebyshev_Sn: Clenshaw, src/detail/Chebyshev.h:135-153)
__host__ __device__ inline void cheb_sn(double x, int n, double *S) {
  const double invn = 1.0 / n;
  for (int m = 0; m < n; ++m) {
    double b1 = 0.0, b2 = 0.0;
    for (int k = n - 1; k >= 1; --k) {
      const double bk = 2 * invn * cos(k * (2.0 * m + 1.0) * (PI / 2) * invn) + 2.0 * x * b1 - b2;
      b2 = b1;
      b1 = bk;
    }
    S[m] = invn + x * b1 - b2;
  }
}

__host__ __device__ inline double cheb_node(int m, int n) { return cos((2.0 * m + 1.0) * PI / (2.0 * n)); }

// The Clenshaw coefficients of S_m (ChebTab, declared with the plan),
// computed once on the host (the same std::cos values as the host-side
// recurrence above) and passed by value, so that no kernel evaluates cos.
inline ChebTab cheb_table(int n) {
  ChebTab t{};
  const double invn = 1.0 / n;
  for (int m = 0; m < n; ++m)
    for (int k = 1; k < n; ++k) t.c[m][k] = 2 * invn * cos(k * (2.0 * m + 1.0) * (PI / 2) * invn);
  return t;
}

// S_m(x), m = 0..n-1, with the tabulated coefficients: the same recurrence
// as cheb_sn.
__device__ __forceinline__ void cheb_sn_tab(double x, int n, const ChebTab &t, double *S) {
  const double invn = 1.0 / n;
  for (int m = 0; m < n; ++m) {
    double b1 = 0.0, b2 = 0.0;
    for (int k = n - 1; k >= 1; --k) {
      const double bk = t.c[m][k] + 2.0 * x * b1 - b2;
      b2 = b1;
      b1 = bk;
    }
    S[m] = invn + x * b1 - b2;
  }
}

// FP32 copy of the Clenshaw coefficients and the same recurrence in FP32
// (mixed-precision P2M and L2P).

inline ChebTab32 cheb_table32(const ChebTab &t) {
  ChebTab32 f{};
  for (int m = 0; m < MAXN_TAB; ++m)
    for (int k = 0; k < MAXN_TAB; ++k) f.c[m][k] = (float)t.c[m][k];
  return f;
}

__device__ __forceinline__ void cheb_sn_tab32(float x, int n, const ChebTab32 &t, float *S) {
  const float invn = 1.0f / (float)n;
  for (int m = 0; m < n; ++m) {
    float b1 = 0.f, b2 = 0.f;
    for (int k = n - 1; k >= 1; --k) {
      const float bk = t.c[m][k] + 2.f * x * b1 - b2;
      b2 = b1;
      b1 = bk;
    }
    S[m] = invn + x * b1 - b2;
  }
}

__host__ __device__ inline double shift_coord(double p, double lo, double hi) {
  const double span = hi - lo;
  return span > 0.0 ? (2 * p - lo - hi) / span : 0.0;
}

template <int KIND> __device__ __forceinline__ double fmm_k64(double d2, double p0) {
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) return exp(-d2 * p0);
  if (KIND == ABX_K_LAPLACE) return 1.0 / (sqrt(d2) + p0);
  if (KIND == ABX_K_MULTIQUADRIC) return sqrt(d2 + p0);
  if (KIND == ABX_K_CONST) return p0;
  return 0.0;
}

template <int KIND> __device__ __forceinline__ float fmm_k32(float d2, float p0) {
  if (KIND == ABX_K_GAUSSIAN || KIND == ABX_K_COMPACT_GAUSSIAN) return __expf(-d2 * p0);
  if (KIND == ABX_K_LAPLACE) return __fdividef(1.0f, sqrtf(d2) + p0);
  if (KIND == ABX_K_MULTIQUADRIC) return sqrtf(d2 + p0);
  if (KIND == ABX_K_CONST) return p0;
  return 0.0f;
}

// ---------------------------------------------------------------- P2M ---
constexpr int FT = 128;
constexpr int MAXN = 8;     // max Chebyshev order
constexpr int MAXC = 512;   // max nodes (8^3)

__global__ void __launch_bounds__(FT) k_p2m(int D, int n, int ncheb, const int *__restrict__ leaves,
                                            const int *__restrict__ nb, const int *__restrict__ ne,
                                            const double *__restrict__ box,
                                            const double *__restrict__ pos, int64_t npos,
                                            const double *__restrict__ b, const int *__restrict__ mi,
                                            const ChebTab tab, double *__restrict__ W) {
  __shared__ double S[FT][MAXN * 3];
  __shared__ double sb[FT];
  const int leaf = leaves[blockIdx.x];
  const double *bx = box + (size_t)leaf * 6;
  double acc[MAXC / FT];
  for (int q = 0; q < MAXC / FT; ++q) acc[q] = 0.0;
  for (int i0 = nb[leaf]; i0 < ne[leaf]; i0 += FT) {
    const int i = i0 + threadIdx.x;
    if (i < ne[leaf]) {
      for (int d = 0; d < D; ++d) {
        const double x = shift_coord(pos[(int64_t)d * npos + i], bx[d], bx[3 + d]);
        cheb_sn_tab(x, n, tab, &S[threadIdx.x][d * MAXN]);
      }
      sb[threadIdx.x] = b[i];
    }
    __syncthreads();
    const int cnt = min(FT, ne[leaf] - i0);
    for (int q = 0; q < MAXC / FT; ++q) {
      const int j = threadIdx.x + q * FT;
      if (j >= ncheb) break;
      double a = 0.0;
      for (int p = 0; p < cnt; ++p) {
        double r = sb[p];
        for (int d = 0; d < D; ++d) r *= S[p][d * MAXN + mi[j * 3 + d]];
        a += r;
      }
      acc[q] += a;
    }
    __syncthreads();
  }
  for (int q = 0; q < MAXC / FT; ++q) {
    const int j = threadIdx.x + q * FT;
    if (j < ncheb) W[(size_t)leaf * ncheb + j] = acc[q];
  }
}

// Mixed-precision P2M: the same sums in FP32 from the leaf-relative FP32
// positions (x = offset / half-width) and FP32 weights; each chunk of FT
// points is summed in FP32 and chunks are added in FP64.
__global__ void __launch_bounds__(FT) k_p2m32(int D, int n, int ncheb, const int *__restrict__ leaves,
                                              const int *__restrict__ nb, const int *__restrict__ ne,
                                              const double *__restrict__ box,
                                              const float4 *__restrict__ posf,
                                              const float *__restrict__ b32,
                                              const int *__restrict__ mi, const ChebTab32 tab,
                                              double *__restrict__ W) {
  __shared__ float S[FT][MAXN * 3 + 1];
  __shared__ float sb[FT];
  __shared__ int smi[MAXC * 3];
  const int leaf = leaves[blockIdx.x];
  const double *bx = box + (size_t)leaf * 6;
  float ihw[3] = {0.f, 0.f, 0.f};
  for (int d = 0; d < D; ++d) {
    const double hw = 0.5 * (bx[3 + d] - bx[d]);
    ihw[d] = hw > 0.0 ? (float)(1.0 / hw) : 0.f;
  }
  for (int e = threadIdx.x; e < ncheb * 3; e += FT) smi[e] = mi[e];
  double acc[MAXC / FT];
  for (int q = 0; q < MAXC / FT; ++q) acc[q] = 0.0;
  for (int i0 = nb[leaf]; i0 < ne[leaf]; i0 += FT) {
    const int i = i0 + threadIdx.x;
    if (i < ne[leaf]) {
      const float4 t = posf[i];
      const float xr[3] = {t.x, t.y, t.z};
      for (int d = 0; d < D; ++d) cheb_sn_tab32(xr[d] * ihw[d], n, tab, &S[threadIdx.x][d * MAXN]);
      sb[threadIdx.x] = b32[i];
    }
    __syncthreads();
    const int cnt = min(FT, ne[leaf] - i0);
    for (int q = 0; q < MAXC / FT; ++q) {
      const int j = threadIdx.x + q * FT;
      if (j >= ncheb) break;
      const int m0 = smi[j * 3], m1 = MAXN + smi[j * 3 + 1], m2 = 2 * MAXN + smi[j * 3 + 2];
      float a = 0.f;
      if (D == 3) {
        for (int p = 0; p < cnt; ++p) a = fmaf(sb[p] * S[p][m0], S[p][m1] * S[p][m2], a);
      } else {
        for (int p = 0; p < cnt; ++p) {
          float r = sb[p];
          for (int d = 0; d < D; ++d) r *= S[p][d * MAXN + smi[j * 3 + d]];
          a += r;
        }
      }
      acc[q] += (double)a;
    }
    __syncthreads();
  }
  for (int q = 0; q < MAXC / FT; ++q) {
    const int j = threadIdx.x + q * FT;
    if (j < ncheb) W[(size_t)leaf * ncheb + j] = acc[q];
  }
}

// ------------------------------------------------------------ M2M / L2L ---
// links: (parent, child, octant), sorted by octant within each level; one CTA
// per (batch of <= NBL links of one level and one octant, FT rows i), so
// that the CTA reads its rows of the octant's ncheb x ncheb matrix once for
// all the batch's links.
// M2M: W[p][i] += sum_j Tc[o][i][j] W[c][j]   (atomic over the parent's
//      children, which other batches hold); read through TcT[o][j][i] =
//      Tc[o][i][j] so that the loads are coalesced along i.
// L2L: G[c][i] += sum_j Tc[o][j][i] G[p][j]   (each child once).
// T is the compute type: double in FP64 mode; float in mixed mode (FP32
// copies of the matrices, FP32 sums of ncheb terms, FP64 storage).
constexpr int NBL = 8;  // links per M2M / L2L batch
template <typename T, bool M2M>
__global__ void __launch_bounds__(FT) k_m2m_l2l(int ncheb, const int *__restrict__ links,
                                                const int2 *__restrict__ batches,
                                                const T *__restrict__ Tm_all,
                                                double *__restrict__ V) {
  const int2 bt = batches[blockIdx.x];
  __shared__ T vin[NBL][MAXC];
  __shared__ int sout[NBL];
  const int o = links[3 * bt.x + 2];
  // M2M reads the children and writes the parents; L2L the other way round
  for (int e = threadIdx.x; e < NBL * ncheb; e += FT) {
    const int b = e / ncheb, j = e - b * ncheb;
    T v = 0;
    if (b < bt.y) {
      const int nd = links[3 * (bt.x + b) + (M2M ? 1 : 0)];
      v = (T)V[(size_t)nd * ncheb + j];
    }
    vin[b][j] = v;
  }
  if (threadIdx.x < bt.y) sout[threadIdx.x] = links[3 * (bt.x + threadIdx.x) + (M2M ? 0 : 1)];
  __syncthreads();
  const T *Tm = Tm_all + (size_t)o * ncheb * ncheb;  // [j][i]
  const int i = blockIdx.y * FT + threadIdx.x;
  if (i < ncheb) {
    T a[NBL];
#pragma unroll
    for (int b = 0; b < NBL; ++b) a[b] = 0;
#pragma unroll 4
    for (int j = 0; j < ncheb; ++j) {
      const T t = Tm[(size_t)j * ncheb + i];
#pragma unroll
      for (int b = 0; b < NBL; ++b) a[b] += t * vin[b][j];
    }
#pragma unroll
    for (int b = 0; b < NBL; ++b) {
      if (b >= bt.y) break;
      double *dst = &V[(size_t)sout[b] * ncheb + i];
      if (M2M) atomicAdd(dst, (double)a[b]);
      else *dst += (double)a[b];
    }
  }
}

// out[o][j][i] = (To)in[o][i][j] (transposed copy of the child matrices).
template <typename To>
__global__ void k_transpose_tc(const double *__restrict__ in, int nchild, int ncheb,
                               To *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)nchild * ncheb * ncheb) return;
  const int64_t o = e / ((int64_t)ncheb * ncheb);
  const int r = (int)(e % ((int64_t)ncheb * ncheb));
  const int j = r / ncheb, i = r % ncheb;
  out[e] = (To)in[(o * ncheb + i) * ncheb + j];
}

// --------------------------------------------------------------- M2L ---
// FP64, one CTA per M2L pair: G[t] += K[m] W[s] (atomic: several sources per
// target run concurrently).
__global__ void __launch_bounds__(FT) k_m2l64(int ncheb, const int *__restrict__ pairs, int npairs,
                                              const double *__restrict__ Km,
                                              const double *__restrict__ W,
                                              double *__restrict__ G) {
  const int q = blockIdx.x;
  if (q >= npairs) return;
  const int t = pairs[3 * q], s = pairs[3 * q + 1], m = pairs[3 * q + 2];
  __shared__ double ws[MAXC];
  for (int j = threadIdx.x; j < ncheb; j += FT) ws[j] = W[(size_t)s * ncheb + j];
  __syncthreads();
  const double *K = Km + (size_t)m * ncheb * ncheb;
  for (int i = threadIdx.x; i < ncheb; i += FT) {
    double a = 0.0;
    for (int j = 0; j < ncheb; ++j) a += K[(size_t)i * ncheb + j] * ws[j];
    atomicAdd(&G[(size_t)t * ncheb + i], a);
  }
}

// Mixed precision M2L on the tensor cores: for one matrix K (ncheb x ncheb,
// FP32) and a tile of 64 (target, source) pairs sharing it:
//   C[16 x 64] (rows i0..i0+15) = K[i0:i0+16, :] * W[:, sources]
// as 3xTF32 (a = ah + al, b = bh + bl; ah*bh + ah*bl + al*bh) on
// mma.sync.m16n8k8.tf32 with FP32 accumulation, then atomically added to G.
__device__ __forceinline__ uint32_t f2tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int TC_PAIRS = 64;  // pairs per CTA

// Split-TF32 parts of the FP32 M2L matrices: hi = tf32(K), lo = tf32(K - hi),
// so that K ~= hi + lo to ~2^-22 and K W ~= hi Wh + hi Wl + lo Wh.
// Rows of ncheb entries are stored with stride ldk (a multiple of 32, zero
// padded), so that the tensor-core kernels stage whole 16-byte-aligned
// 32-column blocks.
__global__ void k_split_tf32(const double *__restrict__ K, int64_t nrows, int ncheb, int ldk,
                             float *__restrict__ hi, float *__restrict__ lo) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nrows * ldk) return;
  const int64_t row = e / ldk;
  const int k = (int)(e % ldk);
  const float f = k < ncheb ? (float)K[row * ncheb + k] : 0.f;
  const uint32_t h = f2tf32(f);
  hi[e] = __uint_as_float(h);
  lo[e] = __uint_as_float(f2tf32(f - __uint_as_float(h)));
}

// W32[node][k] = (float)W[node][k] with row stride ldk (zero padded).
__global__ void k_to_f32_padded(const double *__restrict__ W, int64_t nrows, int ncheb, int ldk,
                                float *__restrict__ W32) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nrows * ldk) return;
  const int64_t row = e / ldk;
  const int k = (int)(e % ldk);
  W32[e] = k < ncheb ? (float)W[row * ncheb + k] : 0.f;
}

// Tensor-core M2L, one CTA per (M2L matrix, 64-pair tile, MT-row block):
// G[tgt_q][rows] += K[rows][:] W[src_q][:] for the tile's pairs q, as an
// MT x 64 x ncheb GEMM in 3xTF32 (mma.sync m16n8k8, FP32 accumulation).
// WM x 2 warps (rows x pairs), 32 x 32 per warp, MT = 32 WM chosen from the
// number of Chebyshev nodes; K and W are staged 32 columns at a time in
// padded shared memory (conflict-free fragment loads); the accumulators
// leave through shared memory as 16-byte vector reductions into G (row
// stride ldg, a multiple of 4).
constexpr int M2_NT = 64, M2_KB = 32, M2_LD = M2_KB + 4;
template <int WM> struct M2Cfg {
  static constexpr int MT = 32 * WM, LDC = MT + 4, THREADS = 64 * WM;
  static constexpr size_t SMEM =
      (size_t)(2 * MT * M2_LD + 2 * M2_NT * M2_LD) * sizeof(float) + 2 * M2_NT * sizeof(int);
  static_assert((size_t)M2_NT * LDC <= (size_t)(2 * MT * M2_LD + 2 * M2_NT * M2_LD),
                "the epilogue tile reuses the staging area");
};

template <int WM>
__global__ void __launch_bounds__(64 * WM) k_m2l_tc2(int ncheb, int ldk, int ldg, const float *__restrict__ Kh,
                                                 const float *__restrict__ Kl,
                                                 const int2 *__restrict__ pairs,
                                                 const int *__restrict__ mat_off,
                                                 const int *__restrict__ tile_mat,
                                                 const int *__restrict__ tile_first,
                                                 const float *__restrict__ W32,
                                                 float *__restrict__ G32) {
  constexpr int M2_MT = M2Cfg<WM>::MT, M2_LDC = M2Cfg<WM>::LDC, NTH = M2Cfg<WM>::THREADS;
  extern __shared__ __align__(16) float m2s[];
  float *sAh = m2s, *sAl = sAh + M2_MT * M2_LD;
  float *sBh = sAl + M2_MT * M2_LD, *sBl = sBh + M2_NT * M2_LD;
  int *sSrc = (int *)(sBl + M2_NT * M2_LD), *sTgt = sSrc + M2_NT;
  float *sC = m2s;  // epilogue, after the main loop
  const int tile = blockIdx.x, i0 = blockIdx.y * M2_MT;
  const int m = tile_mat[tile], p0 = tile_first[tile];
  const int np = min(M2_NT, mat_off[m + 1] - p0);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t4 = lane & 3;
  const int wm = warp % WM, wn = warp / WM;
  if (tid < M2_NT) {
    const int2 pr = tid < np ? pairs[p0 + tid] : make_int2(-1, -1);
    sTgt[tid] = pr.x;
    sSrc[tid] = pr.y;
  }
  const float *Ah = Kh + (size_t)m * ncheb * ldk, *Al = Kl + (size_t)m * ncheb * ldk;
  float c[2][4][4] = {};
  for (int k0 = 0; k0 < ncheb; k0 += M2_KB) {
    __syncthreads();
    for (int e = tid; e < M2_MT * M2_KB; e += NTH) {
      const int r = e / M2_KB, cc = e % M2_KB, i = i0 + r, k = k0 + cc;
      const bool in = i < ncheb && k < ncheb;
      sAh[r * M2_LD + cc] = in ? Ah[(size_t)i * ldk + k] : 0.f;
      sAl[r * M2_LD + cc] = in ? Al[(size_t)i * ldk + k] : 0.f;
    }
    for (int e = tid; e < M2_NT * M2_KB; e += NTH) {
      const int q = e / M2_KB, cc = e % M2_KB, k = k0 + cc;
      const int sidx = sSrc[q];
      const float v = (sidx >= 0 && k < ncheb) ? W32[(size_t)sidx * ldk + k] : 0.f;
      const uint32_t h = f2tf32(v);
      sBh[q * M2_LD + cc] = __uint_as_float(h);
      sBl[q * M2_LD + cc] = __uint_as_float(f2tf32(v - __uint_as_float(h)));
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < M2_KB; kk += 8) {
      uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
      for (int mf = 0; mf < 2; ++mf) {
        const int r = wm * 32 + mf * 16 + g;
        ah[mf][0] = __float_as_uint(sAh[r * M2_LD + kk + t4]);
        ah[mf][1] = __float_as_uint(sAh[(r + 8) * M2_LD + kk + t4]);
        ah[mf][2] = __float_as_uint(sAh[r * M2_LD + kk + t4 + 4]);
        ah[mf][3] = __float_as_uint(sAh[(r + 8) * M2_LD + kk + t4 + 4]);
        al[mf][0] = __float_as_uint(sAl[r * M2_LD + kk + t4]);
        al[mf][1] = __float_as_uint(sAl[(r + 8) * M2_LD + kk + t4]);
        al[mf][2] = __float_as_uint(sAl[r * M2_LD + kk + t4 + 4]);
        al[mf][3] = __float_as_uint(sAl[(r + 8) * M2_LD + kk + t4 + 4]);
      }
#pragma unroll
      for (int nf = 0; nf < 4; ++nf) {
        const int q = wn * 32 + nf * 8 + g;
        bh[nf][0] = __float_as_uint(sBh[q * M2_LD + kk + t4]);
        bh[nf][1] = __float_as_uint(sBh[q * M2_LD + kk + t4 + 4]);
        bl[nf][0] = __float_as_uint(sBl[q * M2_LD + kk + t4]);
        bl[nf][1] = __float_as_uint(sBl[q * M2_LD + kk + t4 + 4]);
      }
#pragma unroll
      for (int mf = 0; mf < 2; ++mf)
#pragma unroll
        for (int nf = 0; nf < 4; ++nf) {
          mma_tf32(c[mf][nf], al[mf], bh[nf]);
          mma_tf32(c[mf][nf], ah[mf], bl[nf]);
          mma_tf32(c[mf][nf], ah[mf], bh[nf]);
        }
    }
  }
  __syncthreads();
  // C fragments -> sC[pair][row]
#pragma unroll
  for (int mf = 0; mf < 2; ++mf)
#pragma unroll
    for (int nf = 0; nf < 4; ++nf) {
      const int r = wm * 32 + mf * 16 + g, q = wn * 32 + nf * 8 + 2 * t4;
      sC[q * M2_LDC + r] = c[mf][nf][0];
      sC[(q + 1) * M2_LDC + r] = c[mf][nf][1];
      sC[q * M2_LDC + r + 8] = c[mf][nf][2];
      sC[(q + 1) * M2_LDC + r + 8] = c[mf][nf][3];
    }
  __syncthreads();
  for (int e = tid; e < M2_NT * (M2_MT / 4); e += NTH) {
    const int q = e / (M2_MT / 4), r4 = (e % (M2_MT / 4)) * 4;
    const int tgt = sTgt[q];
    if (tgt < 0 || i0 + r4 >= ncheb) continue;
    const float4 v = *reinterpret_cast<const float4 *>(&sC[q * M2_LDC + r4]);
    float *dst = G32 + (size_t)tgt * ldg + i0 + r4;  // 16-byte aligned: ldg, i0 + r4 multiples of 4
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(v.x), "f"(v.y),
                 "f"(v.z), "f"(v.w)
                 : "memory");
  }
}

// ------------------------------------------------- M2L on tcgen05 (TMEM) ---
// The same tile GEMM on the 5th-generation tensor cores.  One CTA (4 warps)
// per (M2L matrix, N-pair tile) computes all NRB = ceil(ncheb/128) row
// blocks, so the gathered source expansions of the tile are read once:
//   G[targets][rb*128 + r] += sum_k K[rb*128 + r][k] * W[sources][k]
// as split TF32 (K = Kh + Kl, W = Wh + Wl; Kl Wh + Kh Wl + Kh Wh) on
// tcgen05.mma kind::tf32 into NRB accumulators of 128 x N FP32 in TMEM.
// The K matrices are packed once per plan into the shared-memory image of a
// pipeline stage (k_pack_tf32), so a stage's A operand is one bulk copy on the
// TMA engine (cp.async.bulk, completion counted on the stage's `fullA`
// mbarrier) and bypasses the load/store pipeline; the W rows of the tile's
// sources are gathered 16 bytes per lane with cp.async.  Operands use the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix;
// the descriptor's leading byte offset is the core-matrix stride along K, the
// stride byte offset along rows).
// Roles, with no CTA-wide barrier inside the loop: warp 0 produces (waits for
// the stage's `empty` barrier, issues block p, then waits for block p-LAG's
// W copies, fences them to the async proxy and arrives on `fullB`); lane 0 of
// warp 1 waits for `fullA` and `fullB`, issues the 3 NRB MMAs of the block
// and commits them to `empty`, and after the last block to `accb`; all four
// warps then wait for `accb` and run the epilogue: each reads its 32
// accumulator lanes (rows) with tcgen05.ld and adds them into G with
// reductions that are coalesced along the rows.  Every wait is bounded: on
// timeout the kernel sets *status, skips the epilogue, waits (bounded) for
// its copies and MMAs in flight and still releases its TMEM.  The ring depth
// keeps the CTAs resident on an SM (by shared memory) within the SM's 512
// TMEM columns.
constexpr int T5_KB = 8;
constexpr int T5_PART = 128 * T5_KB * 4;  // bytes of one K operand part: 128 rows x 8 columns
constexpr uint32_t T5_POLL_CAP = 1u << 30;  // second bound on the polls of one wait
// Per row-block count: N pairs per tile, ring depth S, producer lag LAG and
// TMEM columns.  Three or four row blocks use 64-pair tiles so that two CTAs
// share an SM (their latencies overlap); one or two use 128-pair tiles.
template <int NRB> struct T5Cfg {
  static constexpr int N = NRB <= 2 ? 128 : 64;
  static constexpr int S = NRB == 2 ? 4 : 3;  // ring depth
  // the producer signals block p - LAG's W copies after issuing block p
  // (LAG < S: the MMAs of block p - S, which free block p's stage, never wait
  // for a block the producer has not signalled)
  static constexpr int LAG = NRB == 2 ? 2 : 1;
  static constexpr int A_BYTES = NRB * 2 * T5_PART;       // K hi, lo of every row block
  static constexpr int B_PART = N * T5_KB * 4;            // W of the N pairs, one part
  static constexpr int STAGE = A_BYTES + 2 * B_PART;
  static constexpr size_t SMEM = (size_t)S * STAGE + 1024 + 2048;  // + alignment, barriers, indices
  static constexpr uint32_t TCOLS = NRB * N <= 128 ? 128u : (NRB * N <= 256 ? 256u : 512u);
};
constexpr int t5_pairs(int nrb) { return nrb <= 2 ? T5Cfg<1>::N : T5Cfg<3>::N; }
static_assert(T5Cfg<1>::N == T5Cfg<2>::N && T5Cfg<3>::N == T5Cfg<4>::N, "tile width per t5_pairs");
// resident CTAs per SM (bounded by shared memory) x TCOLS <= the SM's 512 TMEM columns
static_assert(T5Cfg<1>::SMEM * 5 > 228 * 1024 && T5Cfg<2>::SMEM * 3 > 228 * 1024 &&
                  T5Cfg<3>::SMEM * 3 > 228 * 1024 && T5Cfg<4>::SMEM * 3 > 228 * 1024,
              "resident CTAs per SM must fit the SM's 512 TMEM columns");
static_assert(T5Cfg<3>::SMEM <= 227 * 1024 && T5Cfg<4>::SMEM <= 227 * 1024, "shared memory per CTA");
static_assert(T5Cfg<1>::LAG < T5Cfg<1>::S && T5Cfg<2>::LAG < T5Cfg<2>::S &&
                  T5Cfg<3>::LAG < T5Cfg<3>::S && T5Cfg<4>::LAG < T5Cfg<4>::S,
              "producer lag below the ring depth");

// Packed split-TF32 M2L matrices: per (matrix, 8-column block kb, 128-row
// block rb, part hi/lo) the 4 KB shared-memory image of the operand tile,
// element (r, k) at ((k/4) * 16 + r/8) * 128 + (r%8) * 16 + (k%4) * 4 bytes;
// zero beyond ncheb.  hi = tf32(K), lo = tf32(K - hi).
__global__ void k_pack_tf32(const double *__restrict__ K, int64_t nmat, int ncheb, int nkb,
                            int nrb, float *__restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nmat * nkb * nrb * 2 * (T5_PART / 4)) return;
  int64_t t = e;
  const int w = (int)(t % (T5_PART / 4));
  t /= T5_PART / 4;
  const int part = (int)(t % 2);
  t /= 2;
  const int rb = (int)(t % nrb);
  t /= nrb;
  const int kb = (int)(t % nkb);
  const int64_t m = t / nkb;
  const int kk = w & 3, rl = (w >> 2) & 7, rh = (w >> 5) & 15, kq = w >> 9;
  const int i = rb * 128 + rh * 8 + rl, k = kb * T5_KB + kq * 4 + kk;
  const float f = (i < ncheb && k < ncheb) ? (float)K[(m * ncheb + i) * ncheb + k] : 0.f;
  const uint32_t h = f2tf32(f);
  out[e] = part == 0 ? __uint_as_float(h) : __uint_as_float(f2tf32(f - __uint_as_float(h)));
}

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor: no swizzle, K-major.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::tf32: D F32, A and B TF32, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for the given phase of an mbarrier for at most limit_ns nanoseconds
// of the GPU's global timer (and at most T5_POLL_CAP polls); false if it ran
// out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
  uint64_t t0 = 0;
  for (uint32_t it = 0; it < T5_POLL_CAP; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((it & 15u) == 0u) {
      const uint64_t now = globaltimer_ns();
      if (it == 0u)
        t0 = now;
      else if (now - t0 > limit_ns)
        return false;
    }
  }
  return false;
}

// 16-byte asynchronous copy; nbytes = 0 writes zeros.
__device__ __forceinline__ void cp16(uint32_t dst, const void *src, int nbytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(nbytes)
               : "memory");
}

template <int NRB>
__global__ void __launch_bounds__(128) k_m2l_tc5(int ncheb, int nkb, int ldk, int ldg,
                                                 const float *__restrict__ Ap,
                                                 const int2 *__restrict__ pairs,
                                                 const int *__restrict__ mat_off,
                                                 const int *__restrict__ tile_mat,
                                                 const int *__restrict__ tile_first,
                                                 const float *__restrict__ Wh,
                                                 const float *__restrict__ Wl,
                                                 float *__restrict__ G32, int *__restrict__ status,
                                                 uint64_t limit_ns, int drop_arrive) {
  using C = T5Cfg<NRB>;
  constexpr int S = C::S, LAG = C::LAG, T5_N = C::N;
  extern __shared__ __align__(128) unsigned char t5raw[];
  unsigned char *sm = (unsigned char *)(((uintptr_t)t5raw + 1023) & ~(uintptr_t)1023);
  uint64_t *fullA = (uint64_t *)(sm + S * C::STAGE);
  uint64_t *fullB = fullA + S, *empty = fullB + S, *accb = empty + S;
  uint32_t *tslot = (uint32_t *)(accb + 1);
  int *sSrc = (int *)(tslot + 4), *sTgt = sSrc + T5_N, *sInfo = sTgt + T5_N;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tile = blockIdx.x;
  const int m = tile_mat[tile], p0 = tile_first[tile];
  const int np = min(T5_N, mat_off[m + 1] - p0);
  if (tid < T5_N) {
    const int2 pr = tid < np ? pairs[p0 + tid] : make_int2(-1, -1);
    sTgt[tid] = pr.x;
    sSrc[tid] = pr.y;
  }
  if (tid == 0) {
    for (int q = 0; q < S; ++q) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&fullA[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&fullB[q])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&empty[q])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(accb)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sInfo[0] = 0;  // blocks issued by the producer
    sInfo[1] = 0;  // blocks whose operands the MMA issuer received
    sInfo[2] = 1;  // producer ok
    sInfo[3] = 1;  // MMA issuer ok
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(tslot)),
                 "r"(C::TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t smbase = smem_addr(sm);

  if (warp == 0) {
    // ---- producer
    const unsigned char *Am = (const unsigned char *)Ap + (size_t)m * nkb * C::A_BYTES;
    bool ok = true;
    int p = 0;
    for (; p < nkb; ++p) {
      const int st = p % S;
      if (p >= S && !mbar_wait(smem_addr(&empty[st]), ((p - S) / S) & 1, limit_ns)) ok = false;
      if (!__all_sync(0xffffffffu, ok)) break;
      const uint32_t sb = smbase + (uint32_t)(st * C::STAGE);
      if (lane == 0) {
        const uint32_t fb = smem_addr(&fullA[st]);
        asm volatile(
            "{\n\t.reg .b64 state;\n\t"
            "mbarrier.arrive.expect_tx.shared::cta.b64 state, [%0], %1;\n\t}" ::"r"(fb),
            "r"(C::A_BYTES)
            : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
            "[%3];" ::"r"(sb),
            "l"(Am + (size_t)p * C::A_BYTES), "r"(C::A_BYTES), "r"(fb)
            : "memory");
      }
#pragma unroll
      for (int e = lane; e < T5_N * (T5_KB / 4); e += 32) {
        const int rl = e & 7, kq = (e >> 3) & 1, rh = e >> 4;
        const int src = sSrc[rh * 8 + rl];
        const uint32_t off = (uint32_t)((kq * (T5_N / 8) + rh) * 128 + rl * 16);
        const size_t g = (size_t)(src >= 0 ? src : 0) * ldk + p * T5_KB + kq * 4;
        cp16(sb + C::A_BYTES + off, Wh + g, src >= 0 ? 16 : 0);
        cp16(sb + C::A_BYTES + C::B_PART + off, Wl + g, src >= 0 ? 16 : 0);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
      if (p >= LAG) {
        // block p - LAG's W copies have landed: hand them to the async proxy
        asm volatile("cp.async.wait_group %0;" ::"n"(LAG) : "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        // drop_arrive (fault injection for tests): block 0's W copies are
        // never signalled, so the MMA issuer's wait runs out
        if (lane == 0 && !(drop_arrive && p - LAG == 0))
          asm volatile("{\n\t.reg .b64 state;\n\tmbarrier.arrive.shared::cta.b64 state, [%0];\n\t}" ::"r"(
                           smem_addr(&fullB[(p - LAG) % S]))
                       : "memory");
      }
    }
    // the last min(p, LAG) blocks
    asm volatile("cp.async.wait_all;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncwarp();
    if (lane == 0) {
      for (int q = max(p - LAG, 0); q < p; ++q)
        if (!(drop_arrive && q == 0))
          asm volatile("{\n\t.reg .b64 state;\n\tmbarrier.arrive.shared::cta.b64 state, [%0];\n\t}" ::"r"(
                         smem_addr(&fullB[q % S]))
                     : "memory");
      sInfo[0] = p;
      if (!ok) sInfo[2] = 0;
    }
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    constexpr uint32_t idesc = umma_idesc_tf32(128, T5_N);
    constexpr uint32_t ks = (128 / 8) * 128;    // core-matrix stride along K (K rows)
    constexpr uint32_t bks = (T5_N / 8) * 128;  // the same for the T5_N pair rows
    bool ok = true;
    int c = 0;
    for (; c < nkb; ++c) {
      const int st = c % S;
      const uint32_t par = (c / S) & 1;
      if (!mbar_wait(smem_addr(&fullA[st]), par, limit_ns) ||
          !mbar_wait(smem_addr(&fullB[st]), par, limit_ns)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smbase + (uint32_t)(st * C::STAGE);
      const uint64_t bh = umma_desc(base + C::A_BYTES, bks, 128);
      const uint64_t bl = umma_desc(base + C::A_BYTES + C::B_PART, bks, 128);
#pragma unroll
      for (int rb = 0; rb < NRB; ++rb) {
        const uint64_t ah = umma_desc(base + rb * 2 * T5_PART, ks, 128);
        const uint64_t al = umma_desc(base + rb * 2 * T5_PART + T5_PART, ks, 128);
        const uint64_t ad[3] = {al, ah, ah}, bd[3] = {bh, bl, bh};
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          const uint32_t acc = (c > 0 || t > 0) ? 1u : 0u;
          asm volatile(
              "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                  tmem + (uint32_t)(rb * T5_N)),
              "l"(ad[t]), "l"(bd[t]), "r"(idesc), "r"(acc));
        }
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_addr(&empty[st])));
    }
    // completes once every MMA issued above has completed
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_addr(accb)));
    sInfo[1] = c;
    if (!ok) sInfo[3] = 0;
  }
  __syncthreads();
  const bool acc_ready = mbar_wait(smem_addr(accb), 0, limit_ns);
  const bool ok = __syncthreads_and(acc_ready && sInfo[2] && sInfo[3] && sInfo[1] == nkb);
  if (!ok) {
    if (tid == 0) {
      atomicExch(status, 1);
      // the MMAs issued so far (accb) and the bulk copies still in flight
      // (fullA) complete before TMEM and shared memory are released; each of
      // these waits is bounded as well
      if (!acc_ready) mbar_wait(smem_addr(accb), 0, limit_ns);
      for (int q = sInfo[1]; q < sInfo[0]; ++q)
        mbar_wait(smem_addr(&fullA[q % S]), (q / S) & 1, limit_ns);
    }
    __syncthreads();
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // per warp a 16 x 32 transpose tile in the (now idle) first stage: lane
    // = row on the way in, (pair, 4 consecutive rows) on the way out, so that
    // G receives 16-byte vector reductions (ldg and the row groups are
    // multiples of 4; groups at or beyond ncheb are skipped)
    float *tt = reinterpret_cast<float *>(sm) + warp * (16 * 32);
#pragma unroll 1
    for (int rb = 0; rb < NRB; ++rb) {
      const int i0 = rb * 128 + 32 * warp;
#pragma unroll 1
      for (int c0 = 0; c0 < T5_N; c0 += 16) {
        uint32_t v[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
              "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
              "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(rb * T5_N + c0)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int q = 0; q < 16; ++q) tt[q * 32 + lane] = __uint_as_float(v[q]);
        __syncwarp();
#pragma unroll
        for (int it = 0; it < 4; ++it) {
          const int q = it * 4 + (lane >> 3), g = (lane & 7) * 4;
          const int tgt = sTgt[c0 + q];
          if (tgt >= 0 && i0 + g < ncheb) {
            const float4 a = *reinterpret_cast<const float4 *>(&tt[q * 32 + g]);
            float *dst = G32 + (size_t)tgt * ldg + i0 + g;
            asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(dst), "f"(a.x),
                         "f"(a.y), "f"(a.z), "f"(a.w)
                         : "memory");
          }
        }
        __syncwarp();
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TCOLS));
}

// G[node][i] += G32[node][i] for the padded FP32 accumulator (row stride ldg).
__global__ void k_add_g32(const float *__restrict__ G32, int64_t nnodes, int ncheb, int ldg,
                          double *__restrict__ G) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnodes * ncheb) return;
  const int64_t node = e / ncheb;
  const int i = (int)(e % ncheb);
  G[e] += (double)G32[node * ldg + i];
}

__global__ void k_f64_to_f32(const double *__restrict__ a, int64_t n, float *__restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// ----------------------------------------------------------- L2P + P2P ---
template <int KIND, bool MIXED>
__global__ void __launch_bounds__(FT) k_l2p_p2p(int D, int n, int ncheb, const int *__restrict__ leaves,
                                                const int *__restrict__ nb,
                                                const int *__restrict__ ne,
                                                const double *__restrict__ box,
                                                const double *__restrict__ pos, int64_t npos,
                                                const double *__restrict__ b,
                                                const int *__restrict__ mi,
                                                const double *__restrict__ G,
                                                const int *__restrict__ rp,
                                                const int *__restrict__ src, double p0,
                                                const ChebTab tab, double *__restrict__ c) {
  __shared__ double sg[MAXC];
  __shared__ double sx[FT], sy[FT], sz[FT], sbv[FT];
  __shared__ int sid[FT];
  const int li = blockIdx.x;
  const int leaf = leaves[li];
  const double *bx = box + (size_t)leaf * 6;
  for (int j = threadIdx.x; j < ncheb; j += FT) sg[j] = G[(size_t)leaf * ncheb + j];
  __syncthreads();
  for (int i0 = nb[leaf]; i0 < ne[leaf]; i0 += FT) {
    const int i = i0 + threadIdx.x;
    const bool act = i < ne[leaf];
    double xi[3] = {0, 0, 0};
    double acc = 0.0;
    if (act) {
      for (int d = 0; d < D; ++d) xi[d] = pos[(int64_t)d * npos + i];
      double S[3][MAXN];
      for (int d = 0; d < D; ++d) cheb_sn_tab(shift_coord(xi[d], bx[d], bx[3 + d]), n, tab, S[d]);
      for (int j = 0; j < ncheb; ++j) {
        double r = sg[j];
        for (int d = 0; d < D; ++d) r *= S[d][mi[j * 3 + d]];
        acc += r;
      }
    }
    // P2P over the connected source leaves
    for (int e = rp[li]; e < rp[li + 1]; ++e) {
      const int sl = src[e];
      for (int j0 = nb[sl]; j0 < ne[sl]; j0 += FT) {
        __syncthreads();
        const int j = j0 + threadIdx.x;
        if (j < ne[sl]) {
          sx[threadIdx.x] = pos[j];
          sy[threadIdx.x] = D > 1 ? pos[npos + j] : 0.0;
          sz[threadIdx.x] = D > 2 ? pos[2 * npos + j] : 0.0;
          sbv[threadIdx.x] = b[j];
          sid[threadIdx.x] = j;
        }
        __syncthreads();
        const int cnt = min(FT, ne[sl] - j0);
        if (act) {
          if (MIXED) {
            // FP32 pair terms summed per staged chunk, chunks summed in FP64;
            // the self pair (a regularised singular kernel can be huge there)
            // is evaluated in FP64.
            float a = 0.f;
            for (int q = 0; q < cnt; ++q) {
              if (sid[q] == i) {
                acc += fmm_k64<KIND>(0.0, p0) * sbv[q];
                continue;
              }
              const float dx = (float)(sx[q] - xi[0]), dy = (float)(sy[q] - xi[1]),
                          dz = (float)(sz[q] - xi[2]);
              const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
              a = fmaf(fmm_k32<KIND>(d2, (float)p0), (float)sbv[q], a);
            }
            acc += (double)a;
          } else {
            for (int q = 0; q < cnt; ++q) {
              const double dx = sx[q] - xi[0], dy = sy[q] - xi[1], dz = sz[q] - xi[2];
              const double d2 = dx * dx + dy * dy + dz * dz;
              acc += fmm_k64<KIND>(d2, p0) * sbv[q];
            }
          }
        }
      }
    }
    if (act) c[i] = acc;
  }
}

// FP32 position of every particle relative to the centre of its leaf: the
// mixed-precision near field works on these small offsets (and on the
// leaf-to-leaf centre offsets), never on absolute FP32 coordinates.
__global__ void k_leaf_rel(int D, const int *__restrict__ leaves, const int *__restrict__ nb,
                           const int *__restrict__ ne, const double *__restrict__ box,
                           const double *__restrict__ pos, int64_t npos,
                           float4 *__restrict__ posf) {
  const int leaf = leaves[blockIdx.x];
  const double *bx = box + (size_t)leaf * 6;
  for (int i = nb[leaf] + threadIdx.x; i < ne[leaf]; i += blockDim.x) {
    float v[3] = {0.f, 0.f, 0.f};
    for (int d = 0; d < D; ++d)
      v[d] = (float)(pos[(int64_t)d * npos + i] - 0.5 * (bx[d] + bx[3 + d]));
    posf[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

__device__ __forceinline__ float rsqrt_approx_f(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_approx_f(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// FP32 kernel value of the mixed near field.  Laplace 1/(|dx| + p0) from the
// hardware reciprocal square root and reciprocal (~2 ulp each): |dx| =
// d2 * rsqrt(d2 + 1e-30), which is 0 at d2 = 0.
template <int KIND> __device__ __forceinline__ float p2p_k32(float d2, float p0) {
  if (KIND == ABX_K_LAPLACE) return rcp_approx_f(fmaf(d2, rsqrt_approx_f(d2 + 1e-30f), p0));
  return fmm_k32<KIND>(d2, p0);
}

constexpr int PT = 32;  // threads per target leaf (one warp) in the mixed near field
constexpr int PW = 4;   // target leaves (warps) per CTA

// Mixed-precision L2P + P2P: one warp per target leaf, one lane per target.
// L2P in FP32 from the leaf-relative FP32 position (x = offset /
// half-width): G of the leaf in FP32, the tensor-product sum nested by
// dimension (the node index is lexicographic, last dimension fastest), the
// innermost two levels in FP32 and the outermost in FP64; each source leaf of the near field is
// staged in shared memory as FP32 offsets from the target leaf's centre
// (leaf-relative FP32 position + FP32 centre offset), the pair terms are FP32
// with a staged chunk (<= 32 terms) summed in FP32 and chunks summed in
// FP64.  The self pair (a regularised singular kernel is huge there) is
// masked out of the FP32 sum and added in FP64.
template <int KIND>
__global__ void __launch_bounds__(PT * PW) k_l2p_p2p32(
    int D, int n, int ncheb, int nleaves, const int *__restrict__ leaves, const int *__restrict__ nb,
    const int *__restrict__ ne, const double *__restrict__ box, const float4 *__restrict__ posf,
    const float *__restrict__ b32, const double *__restrict__ b, const double *__restrict__ G,
    const int *__restrict__ rp, const int *__restrict__ src, double p0, const ChebTab32 tab,
    double *__restrict__ c) {
  __shared__ float sg_all[PW][MAXC];
  __shared__ float4 ss_all[PW][PT];
  __shared__ float sS_all[PW][3][MAXN][PT];  // per-lane Chebyshev values [d][m][lane]
  const int tid = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int li = blockIdx.x * PW + wl;
  if (li >= nleaves) return;  // whole warps: only warp-level synchronisation below
  float *sg = sg_all[wl];
  float4 *ss = ss_all[wl];
  const int leaf = leaves[li];
  const double *bx = box + (size_t)leaf * 6;
  double ct[3] = {0.0, 0.0, 0.0};
  float ihw[3] = {0.f, 0.f, 0.f};
  for (int d = 0; d < D; ++d) {
    ct[d] = 0.5 * (bx[d] + bx[3 + d]);
    const double hw = 0.5 * (bx[3 + d] - bx[d]);
    ihw[d] = hw > 0.0 ? (float)(1.0 / hw) : 0.f;
  }
  for (int j = tid; j < ncheb; j += PT) sg[j] = (float)G[(size_t)leaf * ncheb + j];
  __syncwarp();
  const float p0f = (float)p0;
  for (int i0 = nb[leaf]; i0 < ne[leaf]; i0 += PT) {
    const int i = i0 + tid;
    const bool act = i < ne[leaf];
    double acc = 0.0;
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) {
      t = posf[i];
      const float xr[3] = {t.x, t.y, t.z};
      float S[MAXN];
      for (int d = 0; d < D; ++d) {
        cheb_sn_tab32(xr[d] * ihw[d], n, tab, S);
        for (int m = 0; m < n; ++m) sS_all[wl][d][m][tid] = S[m];
      }
      // sum_{m0} S0 sum_{m1} S1 sum_{m2} S2 g[m0, m1, m2] (D = 3; fewer levels below)
      const float(*sS)[MAXN][PT] = sS_all[wl];
      if (D == 3) {
        for (int m0 = 0; m0 < n; ++m0) {
          float p1 = 0.f;
          for (int m1 = 0; m1 < n; ++m1) {
            const float *gg = sg + (m0 * n + m1) * n;
            float p2 = 0.f;
            for (int m2 = 0; m2 < n; ++m2) p2 = fmaf(gg[m2], sS[2][m2][tid], p2);
            p1 = fmaf(p2, sS[1][m1][tid], p1);
          }
          acc += (double)(p1 * sS[0][m0][tid]);
        }
      } else if (D == 2) {
        for (int m0 = 0; m0 < n; ++m0) {
          float p1 = 0.f;
          for (int m1 = 0; m1 < n; ++m1) p1 = fmaf(sg[m0 * n + m1], sS[1][m1][tid], p1);
          acc += (double)(p1 * sS[0][m0][tid]);
        }
      } else {
        for (int m0 = 0; m0 < n; ++m0) acc += (double)(sg[m0] * sS[0][m0][tid]);
      }
    }
    for (int e = rp[li]; e < rp[li + 1]; ++e) {
      const int sl = src[e];
      const double *sbx = box + (size_t)sl * 6;
      float off[3] = {0.f, 0.f, 0.f};
      for (int d = 0; d < D; ++d) off[d] = (float)(0.5 * (sbx[d] + sbx[3 + d]) - ct[d]);
      const bool own = sl == leaf;
      for (int j0 = nb[sl]; j0 < ne[sl]; j0 += PT) {
        __syncwarp();
        const int j = j0 + tid;
        if (j < ne[sl]) {
          const float4 q = posf[j];
          ss[tid] = make_float4(q.x + off[0], q.y + off[1], q.z + off[2], b32[j]);
        }
        __syncwarp();
        const int cnt = min(PT, ne[sl] - j0);
        if (act) {
          float a = 0.f;
          if (own) {
            for (int q = 0; q < cnt; ++q) {
              const float4 sq = ss[q];
              const float dx = sq.x - t.x, dy = sq.y - t.y, dz = sq.z - t.z;
              const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
              const float w = j0 + q == i ? 0.f : p2p_k32<KIND>(d2, p0f);
              a = fmaf(w, sq.w, a);
            }
            if (i >= j0 && i < j0 + cnt) acc += fmm_k64<KIND>(0.0, p0) * b[i];
          } else {
#pragma unroll 4
            for (int q = 0; q < cnt; ++q) {
              const float4 sq = ss[q];
              const float dx = sq.x - t.x, dy = sq.y - t.y, dz = sq.z - t.z;
              const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
              a = fmaf(p2p_k32<KIND>(d2, p0f), sq.w, a);
            }
          }
          acc += (double)a;
        }
      }
    }
    if (act) c[i] = acc;
  }
}

// M2L matrices: for each (level box size, offset) K[i][j] = kernel(x_i^t, x_j^s)
template <int KIND>
__global__ void k_m2l_mats(int D, int n, int ncheb, const double *__restrict__ mat_desc,
                           const int *__restrict__ mi, double p0, double *__restrict__ Km) {
  // mat_desc per matrix: box size[3], offset[3] (source box lo - target box lo)
  const int m = blockIdx.y;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)ncheb * ncheb) return;
  const int i = (int)(e / ncheb), j = (int)(e % ncheb);
  const double *md = mat_desc + (size_t)m * 6;
  double d2 = 0.0;
  for (int d = 0; d < D; ++d) {
    const double h = md[d];
    const double pi = 0.5 * (cheb_node(mi[i * 3 + d], n) + 1) * h;
    const double pj = 0.5 * (cheb_node(mi[j * 3 + d], n) + 1) * h + md[3 + d];
    const double dx = pj - pi;
    d2 += dx * dx;
  }
  Km[(size_t)m * ncheb * ncheb + e] = fmm_k64<KIND>(d2, p0);
}

}  // namespace

// ----------------------------------------------------------- plan build ---
// eta scales the admissibility of a box pair: it is near (P2P or further
// refinement) iff (max diameter)^2 > eta^2 (box distance)^2; eta = 1 is the
// reference FMM's theta_condition (src/detail/FastMultipoleMethod.h:1249-1279).
int fmm_plan_build(abx_operator *op, int order, FmmPlan *&out, double eta = 1.0) {
  abx_particles *p = op->rows;
  abx_context *ctx = p->ctx;
  cudaStream_t s = ctx->stream;
  ABX_REQUIRE(p->searchable && p->search_kind == 1, ABX_ERR_STATE,
              "the FMM needs an octree: call abx_particles_init_octree first");
  ABX_REQUIRE(order >= 2 && order <= MAXN, ABX_ERR_INVALID, "Chebyshev order must be in 2..%d", MAXN);
  const auto t0 = std::chrono::steady_clock::now();
  const OctTree &T = p->tree;
  FmmPlan *P = new FmmPlan();
  const int D = p->dim;
  P->D = D;
  P->n = order;
  P->tab = cheb_table(order);
  P->tab32 = cheb_table32(P->tab);
  P->nchild = 1 << D;
  P->ncheb = 1;
  for (int d = 0; d < D; ++d) P->ncheb *= order;
  P->kind = op->k.kind;
  P->p0 = op->k.p[0];
  const int nc = P->ncheb;
  P->mi.assign((size_t)nc * 3, 0);
  for (int j = 0; j < nc; ++j) {
    int r = j;
    for (int d = D - 1; d >= 0; --d) {
      P->mi[j * 3 + d] = r % order;
      r /= order;
    }
  }
  const int NN = (int)T.tag.size();
  P->nnodes = NN;
  std::vector<double> boxes((size_t)NN * 6, 0.0);
  for (int nd = 0; nd < NN; ++nd) {
    double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    T.box(p->grid, nd, lo, hi);
    for (int d = 0; d < 3; ++d) {
      boxes[nd * 6 + d] = d < D ? lo[d] : 0.0;
      boxes[nd * 6 + 3 + d] = d < D ? hi[d] : 1.0;
    }
  }
  // ---- traversal on the device: M2L pairs grouped by matrix key, P2P lists
  DevBuf<double> boxes_d;
  if (int e = boxes_d.reserve(boxes.size() + 1)) {
    delete P;
    return e;
  }
  if (!boxes.empty())
    cudaMemcpyAsync(boxes_d.ptr, boxes.data(), boxes.size() * 8, cudaMemcpyHostToDevice, s);
  FmmLists lists;
  if (NN > 1) {
    const int e = fmm_traverse_device(p, boxes_d.ptr, eta, lists);
    if (e != ABX_OK) {
      delete P;
      return e;
    }
  } else {
    lists.mat_off.assign(1, 0);
  }
  // ---- links by level, octant-major (M2M bottom-up uses deepest first)
  std::vector<std::array<int, 3>> links;  // parent, child, octant
  int maxlev = 0;
  {
    const OctDev &O = p->oct;
    for (size_t L = 1; L < O.lvl_base.size(); ++L)
      for (int c = 0; c < O.lvl_count[L]; ++c) {
        const int t = O.lvl_base[L] + c;
        if (T.kind[t] == 0) continue;
        links.push_back({T.parent[t], t, c % P->nchild});
        maxlev = std::max(maxlev, (int)L);
      }
  }
  std::vector<int> flat;
  std::vector<int2> batches;
  P->batch_off.assign(maxlev + 2, 0);
  P->batch_cnt.assign(maxlev + 2, 0);
  {
    std::vector<std::vector<std::vector<int>>> by(maxlev + 1,
                                                  std::vector<std::vector<int>>(P->nchild));
    for (size_t q = 0; q < links.size(); ++q)
      by[T.level[links[q][1]]][links[q][2]].push_back((int)q);
    for (int lev = 1; lev <= maxlev; ++lev) {
      P->batch_off[lev] = (int)batches.size();
      // octant-major within the level: batches of <= NBL links share a matrix
      for (int o = 0; o < P->nchild; ++o) {
        int run = 0;
        for (int q : by[lev][o]) {
          const int idx = (int)(flat.size() / 3);
          if (run == 0) batches.push_back(make_int2(idx, 0));
          ++batches.back().y;
          run = (run + 1) % NBL;
          flat.push_back(links[q][0]);
          flat.push_back(links[q][1]);
          flat.push_back(links[q][2]);
        }
      }
      P->batch_cnt[lev] = (int)batches.size() - P->batch_off[lev];
    }
  }
  // ---- M2L matrices: (level, offset) keys from the traversal, the box size
  // of a representative target
  std::vector<double> mdesc;
  P->nmat = (int)lists.mat_key.size();
  P->n_m2l = (int)lists.n_m2l;
  for (int m = 0; m < P->nmat; ++m) {
    const int t = lists.mat_rep[m];
    double hbox[3] = {1, 1, 1};
    for (int d = 0; d < D; ++d) hbox[d] = boxes[t * 6 + 3 + d] - boxes[t * 6 + d];
    for (int d = 0; d < 3; ++d) mdesc.push_back(hbox[d]);
    for (int d = 0; d < 3; ++d)
      mdesc.push_back(d < D ? (double)lists.mat_key[m][1 + d] * hbox[d] : 0.0);
  }
  P->mat_off = lists.mat_off;
  std::vector<int> leaves = T.leaves;
  P->nleaves = (int)leaves.size();
  // ---- child interpolation matrices Tc[o][i][j] = R_i(node j of child o; parent box)
  std::vector<double> Tc((size_t)P->nchild * nc * nc);
  for (int o = 0; o < P->nchild; ++o)
    for (int j = 0; j < nc; ++j) {
      double S[3][MAXN];
      for (int d = 0; d < D; ++d) {
        const int bit = (o >> (D - 1 - d)) & 1;  // child box in the unit parent box [-1,1]
        const double clo = bit ? 0.0 : -1.0, chi = bit ? 1.0 : 0.0;
        const double x = 0.5 * (cheb_node(P->mi[j * 3 + d], order) + 1) * (chi - clo) + clo;
        cheb_sn(x, order, S[d]);
      }
      for (int i = 0; i < nc; ++i) {
        double r = 1.0;
        for (int d = 0; d < D; ++d) r *= S[d][P->mi[i * 3 + d]];
        Tc[((size_t)o * nc + i) * nc + j] = r;
      }
    }
  // ---- device upload
  int st;
  auto fail = [&](int e) {
    delete P;
    return e;
  };
  std::vector<int> nb(NN), ne(NN);
  for (int nd = 0; nd < NN; ++nd) {
    nb[nd] = T.begin[nd];
    ne[nd] = T.end[nd];
  }
  if ((st = P->W.reserve((size_t)NN * nc)) || (st = P->G.reserve((size_t)NN * nc)) ||
      (st = P->Tc.reserve(Tc.size())) || (st = P->box.reserve(boxes.size())) ||
      (st = P->leaf_ids.reserve(leaves.size() + 1)) || (st = P->node_begin.reserve(NN)) ||
      (st = P->node_end.reserve(NN)) || (st = P->links.reserve(flat.size() + 1)) ||
      (st = P->batches.reserve(batches.size() + 1)) || (st = P->TcT.reserve(Tc.size())) ||
      (st = P->Km.reserve((size_t)std::max(1, P->nmat) * nc * nc)) ||
      (st = P->mat_off_d.reserve(P->nmat + 1)))
    return fail(st);
  // the traversal's device lists move into the plan
  auto take = [](auto &dst, auto &src) {
    std::swap(dst.ptr, src.ptr);
    std::swap(dst.cap, src.cap);
  };
  take(P->m2l, lists.m2l_trip);
  take(P->m2l_by_mat, lists.m2l_by_mat);
  take(P->p2p_rowptr, lists.p2p_rowptr);
  take(P->p2p_src, lists.p2p_src);
  if ((st = P->m2l.reserve(1)) || (st = P->m2l_by_mat.reserve(1)) ||
      (st = P->p2p_rowptr.reserve(1)) || (st = P->p2p_src.reserve(1)))
    return fail(st);
  if (NN <= 1) {
    const int zero = 0;
    cudaMemcpyAsync(P->p2p_rowptr.ptr, &zero, 4, cudaMemcpyHostToDevice, s);
  }
  DevBuf<double> md_d;
  if ((st = P->mi_d.reserve(P->mi.size())) || (st = md_d.reserve(mdesc.size() + 1))) return fail(st);
  // tensor-core M2L tiles: 64 pairs for the mma.sync kernel (<= 64 nodes),
  // t5_pairs pairs for the tcgen05 kernel, of one matrix each
  std::vector<int> tmat, tfirst;
  const int tile_pairs = nc <= 64 ? TC_PAIRS : t5_pairs((nc + 127) / 128);
  for (int m = 0; m < P->nmat; ++m)
    for (int q = P->mat_off[m]; q < P->mat_off[m + 1]; q += tile_pairs) {
      tmat.push_back(m);
      tfirst.push_back(q);
    }
  P->ntiles = (int)tmat.size();
  if ((st = P->tile_mat.reserve(tmat.size() + 1)) || (st = P->tile_first.reserve(tfirst.size() + 1)))
    return fail(st);
  auto up = [&](void *dst, const void *src, size_t bytes) {
    if (bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  up(P->Tc.ptr, Tc.data(), Tc.size() * 8);
  if (!Tc.empty())
    k_transpose_tc<double><<<ceil_div(Tc.size(), 256), 256, 0, s>>>(P->Tc.ptr, P->nchild, nc,
                                                                   P->TcT.ptr);
  up(P->box.ptr, boxes.data(), boxes.size() * 8);
  up(P->leaf_ids.ptr, leaves.data(), leaves.size() * 4);
  up(P->node_begin.ptr, nb.data(), nb.size() * 4);
  up(P->node_end.ptr, ne.data(), ne.size() * 4);
  up(P->links.ptr, flat.data(), flat.size() * 4);
  up(P->batches.ptr, batches.data(), batches.size() * sizeof(int2));
  up(P->mat_off_d.ptr, P->mat_off.data(), P->mat_off.size() * 4);
  up(P->mi_d.ptr, P->mi.data(), P->mi.size() * 4);
  up(P->tile_mat.ptr, tmat.data(), tmat.size() * 4);
  up(P->tile_first.ptr, tfirst.data(), tfirst.size() * 4);
  up(md_d.ptr, mdesc.data(), mdesc.size() * 8);
  if (P->nmat > 0) {
    dim3 grid(ceil_div((size_t)nc * nc, 256), P->nmat);
    switch (P->kind) {
    case ABX_K_LAPLACE: k_m2l_mats<ABX_K_LAPLACE><<<grid, 256, 0, s>>>(D, order, nc, md_d.ptr, P->mi_d.ptr, P->p0, P->Km.ptr); break;
    case ABX_K_GAUSSIAN: k_m2l_mats<ABX_K_GAUSSIAN><<<grid, 256, 0, s>>>(D, order, nc, md_d.ptr, P->mi_d.ptr, P->p0, P->Km.ptr); break;
    case ABX_K_COMPACT_GAUSSIAN: k_m2l_mats<ABX_K_COMPACT_GAUSSIAN><<<grid, 256, 0, s>>>(D, order, nc, md_d.ptr, P->mi_d.ptr, P->p0, P->Km.ptr); break;
    case ABX_K_MULTIQUADRIC: k_m2l_mats<ABX_K_MULTIQUADRIC><<<grid, 256, 0, s>>>(D, order, nc, md_d.ptr, P->mi_d.ptr, P->p0, P->Km.ptr); break;
    case ABX_K_CONST: k_m2l_mats<ABX_K_CONST><<<grid, 256, 0, s>>>(D, order, nc, md_d.ptr, P->mi_d.ptr, P->p0, P->Km.ptr); break;
    default:
      set_error("FMM: kernel kind %d not supported", P->kind);
      return fail(ABX_ERR_INVALID);
    }
  }
  if (P->nleaves > 0) {
    if ((st = P->posf.reserve((size_t)std::max<int64_t>(op->rows->n, 1)))) return fail(st);
    k_leaf_rel<<<P->nleaves, FT, 0, s>>>(D, P->leaf_ids.ptr, P->node_begin.ptr, P->node_end.ptr,
                                          P->box.ptr, op->rows->pos.ptr, op->rows->n, P->posf.ptr);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    set_error("FMM plan upload failed");
    return fail(ABX_ERR_CUDA);
  }
  P->max_level.assign(1, maxlev);
  P->build_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  out = P;
  return ABX_OK;
}

namespace {
template <int KIND>
int launch_l2p_p2p(FmmPlan *P, cudaStream_t s, const double *pos, int64_t npos, const double *b,
                   double *c, bool mixed) {
  if (mixed) {
    // P->b32 holds this matvec's FP32 weights (converted before the P2M)
    k_l2p_p2p32<KIND><<<ceil_div((size_t)P->nleaves, PW), PT * PW, 0, s>>>(
        P->D, P->n, P->ncheb, P->nleaves, P->leaf_ids.ptr, P->node_begin.ptr, P->node_end.ptr,
        P->box.ptr, P->posf.ptr, P->b32.ptr, b, P->G.ptr, P->p2p_rowptr.ptr, P->p2p_src.ptr,
        P->p0, P->tab32, c);
  } else
    k_l2p_p2p<KIND, false><<<P->nleaves, FT, 0, s>>>(
        P->D, P->n, P->ncheb, P->leaf_ids.ptr, P->node_begin.ptr, P->node_end.ptr, P->box.ptr, pos,
        npos, b, P->mi_d.ptr, P->G.ptr, P->p2p_rowptr.ptr, P->p2p_src.ptr, P->p0, P->tab, c);
  ABX_CHECK_CUDA(cudaGetLastError());
  return ABX_OK;
}
}  // namespace

// c = K b through the five FMM passes (storage order of the octree set).
int fmm_matvec_device(abx_operator *op, const double *b, double *c) {
  FmmPlan *P = op->fmm;
  abx_particles *p = op->rows;
  cudaStream_t s = p->ctx->stream;
  const int nc = P->ncheb;
  const int64_t npos = p->n;
  if (npos == 0) return ABX_OK;
  const bool mixed = op->precision == ABX_PREC_MIXED;
  ABX_CHECK_CUDA(cudaMemsetAsync(P->W.ptr, 0, (size_t)P->nnodes * nc * 8, s));
  ABX_CHECK_CUDA(cudaMemsetAsync(P->G.ptr, 0, (size_t)P->nnodes * nc * 8, s));
  if (mixed) {
    ABX_TRY(P->b32.reserve((size_t)npos));
    k_f64_to_f32<<<ceil_div((size_t)npos, 256), 256, 0, s>>>(b, npos, P->b32.ptr);
    if (!P->Tc32.ptr) {
      const size_t nt = (size_t)P->nchild * nc * nc;
      ABX_TRY(P->Tc32.reserve(nt));
      ABX_TRY(P->Tc32T.reserve(nt));
      k_f64_to_f32<<<ceil_div(nt, 256), 256, 0, s>>>(P->Tc.ptr, nt, P->Tc32.ptr);
      k_transpose_tc<float><<<ceil_div(nt, 256), 256, 0, s>>>(P->Tc.ptr, P->nchild, nc,
                                                             P->Tc32T.ptr);
    }
  }
  if (P->nleaves > 0) {
    if (mixed)
      k_p2m32<<<P->nleaves, FT, 0, s>>>(P->D, P->n, nc, P->leaf_ids.ptr, P->node_begin.ptr,
                                        P->node_end.ptr, P->box.ptr, P->posf.ptr, P->b32.ptr,
                                        P->mi_d.ptr, P->tab32, P->W.ptr);
    else
      k_p2m<<<P->nleaves, FT, 0, s>>>(P->D, P->n, nc, P->leaf_ids.ptr, P->node_begin.ptr,
                                      P->node_end.ptr, P->box.ptr, p->pos.ptr, npos, b,
                                      P->mi_d.ptr, P->tab, P->W.ptr);
  }
  const int maxlev = P->max_level.empty() ? 0 : P->max_level[0];
  for (int lev = maxlev; lev >= 1; --lev)
    if (P->batch_cnt[lev] > 0) {
      const int2 *bt = P->batches.ptr + P->batch_off[lev];
      if (mixed)
        k_m2m_l2l<float, true><<<dim3(P->batch_cnt[lev], ceil_div(nc, FT)), FT, 0, s>>>(nc, P->links.ptr, bt,
                                                              P->Tc32T.ptr, P->W.ptr);
      else
        k_m2m_l2l<double, true><<<dim3(P->batch_cnt[lev], ceil_div(nc, FT)), FT, 0, s>>>(nc, P->links.ptr, bt,
                                                               P->TcT.ptr, P->W.ptr);
    }
  ABX_CHECK_CUDA(cudaGetLastError());
  if (P->n_m2l > 0) {
    if (mixed) {
      const size_t tot = (size_t)P->nnodes * nc;
      const int ldg = (nc + 3) / 4 * 4;
      const int ldk = (nc + 31) / 32 * 32;
      ABX_TRY(P->W32.reserve((size_t)P->nnodes * ldk));
      ABX_TRY(P->G32.reserve((size_t)P->nnodes * ldg));
      ABX_CHECK_CUDA(cudaMemsetAsync(P->G32.ptr, 0, (size_t)P->nnodes * ldg * 4, s));
      if (nc <= 64) {
        // mma.sync tiles (a 128-row tcgen05 tile would be mostly padding)
        if (!P->Kmh.ptr) {
          const size_t nk = (size_t)P->nmat * nc * ldk;
          ABX_TRY(P->Kmh.reserve(nk));
          ABX_TRY(P->Kml.reserve(nk));
          k_split_tf32<<<ceil_div(nk, 256), 256, 0, s>>>(P->Km.ptr, (int64_t)P->nmat * nc, nc,
                                                         ldk, P->Kmh.ptr, P->Kml.ptr);
        }
        k_to_f32_padded<<<ceil_div((size_t)P->nnodes * ldk, 256), 256, 0, s>>>(
            P->W.ptr, P->nnodes, nc, ldk, P->W32.ptr);
        auto launch_m2l = [&](auto kern, int mt, int threads, size_t smem) -> int {
          ABX_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
          const dim3 grid(P->ntiles, (nc + mt - 1) / mt);
          kern<<<grid, threads, smem, s>>>(nc, ldk, ldg, P->Kmh.ptr, P->Kml.ptr,
                                           P->m2l_by_mat.ptr, P->mat_off_d.ptr, P->tile_mat.ptr,
                                           P->tile_first.ptr, P->W32.ptr, P->G32.ptr);
          return ABX_OK;
        };
        if (nc <= 32)
          ABX_TRY(launch_m2l(k_m2l_tc2<1>, M2Cfg<1>::MT, M2Cfg<1>::THREADS, M2Cfg<1>::SMEM));
        else
          ABX_TRY(launch_m2l(k_m2l_tc2<2>, M2Cfg<2>::MT, M2Cfg<2>::THREADS, M2Cfg<2>::SMEM));
      } else {
        // 5th-generation tensor cores (tcgen05, TMEM accumulators)
        const int nkb = (nc + T5_KB - 1) / T5_KB;
        const int nrb = (nc + 127) / 128;  // 1..4 for orders 5..8
        if (!P->Kp.ptr) {
          const size_t nk = (size_t)P->nmat * nkb * nrb * 2 * (T5_PART / 4);
          ABX_TRY(P->Kp.reserve(nk));
          k_pack_tf32<<<ceil_div(nk, 256), 256, 0, s>>>(P->Km.ptr, P->nmat, nc, nkb, nrb,
                                                        P->Kp.ptr);
        }
        ABX_TRY(P->W32l.reserve((size_t)P->nnodes * ldk));
        k_split_tf32<<<ceil_div((size_t)P->nnodes * ldk, 256), 256, 0, s>>>(
            P->W.ptr, P->nnodes, nc, ldk, P->W32.ptr, P->W32l.ptr);
        int *status = p->ctx->dev_flag.ptr + 8;
        ABX_CHECK_CUDA(cudaMemsetAsync(status, 0, sizeof(int), s));
        auto launch_tc5 = [&](auto kern, size_t smem) -> int {
          ABX_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
          kern<<<P->ntiles, 128, smem, s>>>(nc, nkb, ldk, ldg, P->Kp.ptr, P->m2l_by_mat.ptr,
                                            P->mat_off_d.ptr, P->tile_mat.ptr, P->tile_first.ptr,
                                            P->W32.ptr, P->W32l.ptr, P->G32.ptr, status,
                                            (uint64_t)(P->wait_limit_s * 1e9), P->drop_arrive);
          return ABX_OK;
        };
        switch (nrb) {
          case 1: ABX_TRY(launch_tc5(k_m2l_tc5<1>, T5Cfg<1>::SMEM)); break;
          case 2: ABX_TRY(launch_tc5(k_m2l_tc5<2>, T5Cfg<2>::SMEM)); break;
          case 3: ABX_TRY(launch_tc5(k_m2l_tc5<3>, T5Cfg<3>::SMEM)); break;
          default: ABX_TRY(launch_tc5(k_m2l_tc5<4>, T5Cfg<4>::SMEM)); break;
        }
        ABX_CHECK_CUDA(cudaGetLastError());
        int st = 0;
        ABX_CHECK_CUDA(cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s));
        ABX_CHECK_CUDA(cudaStreamSynchronize(s));
        ABX_REQUIRE(st == 0, ABX_ERR_TIMEOUT, "FMM M2L: a tensor-core completion wait timed out");
      }
      k_add_g32<<<ceil_div(tot, 256), 256, 0, s>>>(P->G32.ptr, P->nnodes, nc, ldg, P->G.ptr);
    } else {
      k_m2l64<<<P->n_m2l, FT, 0, s>>>(nc, P->m2l.ptr, P->n_m2l, P->Km.ptr, P->W.ptr, P->G.ptr);
    }
    ABX_CHECK_CUDA(cudaGetLastError());
  }
  for (int lev = 1; lev <= maxlev; ++lev)
    if (P->batch_cnt[lev] > 0) {
      const int2 *bt = P->batches.ptr + P->batch_off[lev];
      if (mixed)
        k_m2m_l2l<float, false><<<dim3(P->batch_cnt[lev], ceil_div(nc, FT)), FT, 0, s>>>(nc, P->links.ptr, bt,
                                                               P->Tc32.ptr, P->G.ptr);
      else
        k_m2m_l2l<double, false><<<dim3(P->batch_cnt[lev], ceil_div(nc, FT)), FT, 0, s>>>(nc, P->links.ptr, bt,
                                                                P->Tc.ptr, P->G.ptr);
    }
  ABX_CHECK_CUDA(cudaGetLastError());
  if (P->nleaves == 0) return ABX_OK;
  switch (P->kind) {
  case ABX_K_LAPLACE: return launch_l2p_p2p<ABX_K_LAPLACE>(P, s, p->pos.ptr, npos, b, c, mixed);
  case ABX_K_GAUSSIAN: return launch_l2p_p2p<ABX_K_GAUSSIAN>(P, s, p->pos.ptr, npos, b, c, mixed);
  case ABX_K_COMPACT_GAUSSIAN:
    return launch_l2p_p2p<ABX_K_COMPACT_GAUSSIAN>(P, s, p->pos.ptr, npos, b, c, mixed);
  case ABX_K_MULTIQUADRIC:
    return launch_l2p_p2p<ABX_K_MULTIQUADRIC>(P, s, p->pos.ptr, npos, b, c, mixed);
  case ABX_K_CONST: return launch_l2p_p2p<ABX_K_CONST>(P, s, p->pos.ptr, npos, b, c, mixed);
  }
  set_error("FMM: unsupported kernel");
  return ABX_ERR_INVALID;
}

}  // namespace abx

using namespace abx;

extern "C" int abx_create_fmm_operator(abx_particles *p, const abx_kernel *k, int order,
                                       abx_operator **out) {
  ABX_REQUIRE(p && k && out, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(k->kind == ABX_K_LAPLACE || k->kind == ABX_K_GAUSSIAN ||
                  k->kind == ABX_K_COMPACT_GAUSSIAN || k->kind == ABX_K_MULTIQUADRIC ||
                  k->kind == ABX_K_CONST,
              ABX_ERR_INVALID, "FMM: kernel kind %d not supported", k->kind);
  ABX_TRY(ctx_activate(p->ctx));
  abx_operator *op = new abx_operator();
  op->kind = 2;
  op->rows = p;
  op->cols = p;
  op->k = *k;
  FmmPlan *P = nullptr;
  const int st = fmm_plan_build(op, order, P);
  if (st != ABX_OK) {
    delete op;
    return st;
  }
  op->fmm = P;
  particles_retain(p);
  particles_retain(p);
  *out = op;
  return ABX_OK;
}

extern "C" int abx_create_h2_operator(abx_particles *p, const abx_kernel *k, int order,
                                      double eta, abx_operator **out) {
  ABX_REQUIRE(p && k && out, ABX_ERR_INVALID, "null argument");
  ABX_REQUIRE(eta > 0.0 && std::isfinite(eta), ABX_ERR_INVALID, "eta must be positive");
  ABX_REQUIRE(k->kind == ABX_K_LAPLACE || k->kind == ABX_K_GAUSSIAN ||
                  k->kind == ABX_K_COMPACT_GAUSSIAN || k->kind == ABX_K_MULTIQUADRIC ||
                  k->kind == ABX_K_CONST,
              ABX_ERR_INVALID, "H2: kernel kind %d not supported", k->kind);
  ABX_TRY(ctx_activate(p->ctx));
  abx_operator *op = new abx_operator();
  op->kind = 2;
  op->rows = p;
  op->cols = p;
  op->k = *k;
  FmmPlan *P = nullptr;
  const int st = fmm_plan_build(op, order, P, eta);
  if (st != ABX_OK) {
    delete op;
    return st;
  }
  op->fmm = P;
  particles_retain(p);
  particles_retain(p);
  *out = op;
  return ABX_OK;
}

extern "C" int abx_fmm_stats(abx_operator *op, int64_t *m2l_pairs, int64_t *matrices,
                             int64_t *leaves, double *plan_seconds) {
  ABX_REQUIRE(op && op->kind == 2 && op->fmm, ABX_ERR_INVALID, "not an FMM operator");
  if (m2l_pairs) *m2l_pairs = op->fmm->n_m2l;
  if (matrices) *matrices = op->fmm->nmat;
  if (leaves) *leaves = op->fmm->nleaves;
  if (plan_seconds) *plan_seconds = op->fmm->build_s;
  return ABX_OK;
}

extern "C" int abx_fmm_set_wait_limit(abx_operator *op, double seconds, int drop_one_arrive) {
  ABX_REQUIRE(op && op->kind == 2 && op->fmm, ABX_ERR_INVALID, "not an FMM operator");
  ABX_REQUIRE(seconds > 0.0 && seconds <= 60.0, ABX_ERR_INVALID,
              "wait limit must be in (0, 60] seconds");
  op->fmm->wait_limit_s = seconds;
  op->fmm->drop_arrive = drop_one_arrive ? 1 : 0;
  return ABX_OK;
}
