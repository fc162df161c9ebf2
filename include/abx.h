/*
 * abx.h -- C ABI of the aboria_gb300 library: the GB300 (sm_103a) particle
 * hot path behind Aboria's header API.
 *
 * Plain C: opaque handles, pointers and sizes, int status codes.  Every entry
 * point returns ABX_OK (0) or an ABX_ERR_* code and leaves a message for
 * abx_last_error().  The reference reports errors with CHECK/ASSERT, which
 * print and raise SIGTRAP (src/Log.h:43-81); the C++ header layer
 * (include/aboria_gb/Aboria.h) maps a non-zero status back to that behaviour.
 *
 * Vector arguments (positions, b, c, counts, ...) may be host memory
 * (pageable or pinned) or device memory of the context's GPU (device memory
 * of another GPU is rejected with ABX_ERR_INVALID); the library detects which
 * (cudaPointerGetAttributes) and stages host buffers through the device
 * around the call.  All work runs on the context's stream; calls that return
 * data to host memory synchronise that stream before returning.
 *
 * Index conventions follow the reference: after
 * abx_particles_init_neighbour_search the particle storage is in cell order
 * (src/Particles.h:694-726), and row/column k of every operator is the k-th
 * particle in that order.  abx_particles_get_ids maps it back to insertion ids.
 */
#ifndef ABX_H_
#define ABX_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ABX_API __attribute__((visibility("default")))
#else
#define ABX_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define ABX_OK 0
#define ABX_ERR_INVALID 1   /* bad argument */
#define ABX_ERR_CUDA 2      /* CUDA runtime error */
#define ABX_ERR_ALLOC 3     /* device allocation failed */
#define ABX_ERR_STATE 4     /* e.g. neighbour search not initialised */
#define ABX_ERR_TIMEOUT 5   /* a bounded device-side wait gave up */
#define ABX_ERR_CAPACITY 6  /* caller-provided output too small */
#define ABX_ERR_NUMERIC 7   /* breakdown / non-finite value detected */

/* Precision modes of the pair kernels. */
#define ABX_PREC_FP64 0  /* FP64 evaluation and accumulation (1e-12 parity mode) */
#define ABX_PREC_MIXED 1 /* FP32 evaluation, FP32 blocks of <=32 terms summed in FP64 */

/* Built-in kernel functors (the closures passed to create_*_operator). */
#define ABX_K_CONST 0            /* p0                                   */
#define ABX_K_GAUSSIAN 1         /* exp(-|dx|^2 * p0)                    */
#define ABX_K_WENDLAND_C2 2      /* q=|dx|*p0: (1-q)^4 (4q+1), 0 if q>=1 */
#define ABX_K_COMPACT_GAUSSIAN 3 /* exp(-p0 |dx|^2), p0 = eps^2          */
#define ABX_K_LAPLACE 4          /* 1/(|dx| + p0)                        */
#define ABX_K_MULTIQUADRIC 5     /* sqrt(|dx|^2 + p0)                    */
#define ABX_K_SCALAR_SUM 6       /* s_row[i] + s_col[j] (particle scalars) */

typedef struct abx_kernel {
  int kind;
  double p[4];
} abx_kernel;

typedef struct abx_context abx_context;
typedef struct abx_particles abx_particles;
typedef struct abx_operator abx_operator;

/* ------------------------------------------------------------ library ---- */
ABX_API const char *abx_last_error(void);
ABX_API int abx_version(void);

/* Execution context: one device and one stream.  stream may be NULL (the
 * library creates its own) or a cudaStream_t owned by the caller. */
ABX_API int abx_context_create(int device, void *stream, abx_context **out);
ABX_API int abx_context_destroy(abx_context *ctx);
ABX_API int abx_context_synchronize(abx_context *ctx);

/* -------------------------------------------------------------- particles --
 * Particles<std::tuple<...>, D> storage (src/Particles.h:108-112): positions
 * (D doubles each, D in 1..3), ids, and one optional scalar column that the
 * ABX_K_SCALAR_SUM functor reads (get<var>(particle) in the reference).      */
ABX_API int abx_particles_create(abx_context *ctx, int dim, abx_particles **out);
ABX_API int abx_particles_destroy(abx_particles *p);
/* Replace the contents with n particles (AoS n*dim positions).  ids may be
 * NULL (ids 0..n-1), like consecutive push_back calls. */
ABX_API int abx_particles_set(abx_particles *p, int64_t n, const double *pos, const int64_t *ids);
/* Per-particle scalar in the current storage order (reordered with the rest). */
ABX_API int abx_particles_set_scalar(abx_particles *p, const double *s);
ABX_API int64_t abx_particles_size(const abx_particles *p);
ABX_API int abx_particles_get_positions(abx_particles *p, double *pos_out);
ABX_API int abx_particles_get_ids(abx_particles *p, int64_t *ids_out);
ABX_API int abx_particles_get_scalar(abx_particles *p, double *s_out);

/* Particles::init_neighbour_search (src/Particles.h:445-456): set the domain,
 * enforce it (periodic wrap or delete, src/NeighbourSearchBase.h:185-238),
 * build the CellListOrdered grid (src/CellListOrdered.h:132-259) and reorder
 * storage into stable (cell key, insertion) order. */
ABX_API int abx_particles_init_neighbour_search(abx_particles *p, const double *lo, const double *hi,
                                        const int *periodic, double n_particles_in_leaf);
/* Particles::update_positions (src/Particles.h:526-540) after positions were
 * replaced with abx_particles_set_positions (same n, current storage order). */
ABX_API int abx_particles_set_positions(abx_particles *p, const double *pos);
ABX_API int abx_particles_update_positions(abx_particles *p);
/* Particles::push_back (src/Particles.h:264-311): append n_new particles (AoS
 * positions) with the next ids (written to ids_out when not NULL); on a
 * searchable set the search structure is updated at once (the reference
 * updates an ordered search after every push_back). */
ABX_API int abx_particles_push_back(abx_particles *p, int64_t n_new, const double *pos,
                                    int64_t *ids_out);
/* Particles::erase(first, last) (src/Particles.h:361-389): the particles at
 * storage positions [first, last) are marked dead and the search structure is
 * updated, which drops them (without a search structure they are removed and
 * the rest keep their order). */
ABX_API int abx_particles_erase(abx_particles *p, int64_t first, int64_t last);
/* Find-by-id (NeighbourSearchBase::find_id_map and find,
 * src/NeighbourSearchBase.h:276-321, 720): the storage index of every id in
 * ids[nq] (host or device memory), -1 for an id not in the set.  The id map
 * (ids sorted, with their storage index) is built on the device on first use
 * after the particles changed. */
ABX_API int abx_particles_find_ids(abx_particles *p, int64_t nq, const int64_t *ids,
                                   int64_t *index_out);
/* Particles<..., HyperOctree>::init_neighbour_search (src/OctTree.h:168-226):
 * domain enforcement as above, then storage reordered by octree tag
 * (src/detail/SpatialUtil.h:255-286, stable) and the tree built level by level
 * with leaves of <= n_particles_in_leaf particles (src/OctTree.h:328-475).
 * The radius search and the operators work on either search structure. */
ABX_API int abx_particles_init_octree(abx_particles *p, const double *lo, const double *hi,
                                      const int *periodic, double n_particles_in_leaf);
/* Leaves of the octree in the reference's creation order (level by level):
 * level, tag, and the [begin, end) range in storage order.  Pass NULL arrays
 * to query *nleaves only. */
ABX_API int abx_particles_get_tree_leaves(abx_particles *p, int64_t *nleaves, int32_t *level,
                                          int32_t *tag, int32_t *begin, int32_t *end,
                                          int64_t cap);
/* Grid of the cell list: size[dim], side[dim], total bucket count. */
ABX_API int abx_particles_get_grid(abx_particles *p, uint32_t *size, double *side, uint32_t *ncells);
/* bucket_begin/bucket_end (src/CellListOrdered.h:231-239), ncells each, and
 * the sorted bucket key of every particle (n). */
ABX_API int abx_particles_get_buckets(abx_particles *p, uint32_t *bucket_begin, uint32_t *bucket_end,
                              uint32_t *keys);

/* Device view of a particle set, for kernels compiled in the caller's
 * translation unit (the C++ header's user-functor operators): plain device
 * pointers into the library's storage, valid until the set is next changed
 * (set, init_neighbour_search, update_positions) or destroyed.  Positions are
 * SoA (pos[d*n + i]); the bucket ranges and grid are the CellListOrdered ones
 * (src/CellListOrdered.h:132-259; bucket key = sum_d v_d prod_{e>d} size_e,
 * v_d the bucket coordinate), NULL for an octree (search_kind 1).  The
 * reference's query object exposes the same data to its search iterators
 * (CellListOrderedQuery, src/CellListOrdered.h:280-491). */
typedef struct abx_particles_view {
  int64_t n;
  int dim;
  int device;
  const double *pos;
  const int64_t *ids;
  const uint32_t *bucket_begin, *bucket_end;
  uint32_t ncells;
  uint32_t size[3];
  double lo[3], hi[3], side[3];
  int periodic[3];
  int search_kind;
} abx_particles_view;
ABX_API int abx_particles_get_view(abx_particles *p, abx_particles_view *out);

/* -------------------------------------------------------- radius search --
 * euclidean_search(query, x, r) (src/Search.h:839-845) for nq query points:
 * every stored particle j (and periodic image) with
 * ((0+dx0^2)+dx1^2)+dx2^2 <= r^2 in FP64, dx = x_j - (x + image*L). */
ABX_API int abx_radius_count(abx_particles *p, int64_t nq, const double *q, double r, int32_t *counts);
/* Neighbour lists as CSR: rowptr[nq+1] and cols[] (indices into storage
 * order; the order within a row is unspecified -- the neighbour set is the
 * reference's, bit for bit, not its visiting order; a particle reached through
 * two periodic images appears twice).  Call with cols == NULL to get rowptr only (nnz in
 * rowptr[nq]); cap is the capacity of cols. */
ABX_API int abx_radius_query_csr(abx_particles *p, int64_t nq, const double *q, double r,
                         int64_t *rowptr, int32_t *cols, int64_t cap);
/* abx_radius_query_csr plus dx[nnz*dim]: for every neighbour the separation
 * x_j - (x + image*L) of the periodic image the search accepted, in FP64 as
 * the reference's search iterator computes it (src/Search.h:188-190, 443). */
ABX_API int abx_radius_query_csr_dx(abx_particles *p, int64_t nq, const double *q, double r,
                                    int64_t *rowptr, int32_t *cols, double *dx, int64_t cap);
/* The same searches in another norm: manhatten_search (lnorm = 1) and
 * chebyshev_search (lnorm = -1), src/Search.h:797-845, with the reference's
 * FP64 test distance_helper<1/-1> (src/detail/Distance.h:46-137): accum = 0,
 * then |dx_d| over the dimensions in order, summed (1) or as a running
 * maximum (-1); a particle is a neighbour iff !(accum > |r|).  lnorm = 2 is
 * euclidean_search (abx_radius_count / abx_radius_query_csr). */
ABX_API int abx_radius_count_lnorm(abx_particles *p, int64_t nq, const double *q, double r,
                                   int lnorm, int32_t *counts);
ABX_API int abx_radius_query_csr_lnorm(abx_particles *p, int64_t nq, const double *q, double r,
                                       int lnorm, int64_t *rowptr, int32_t *cols, int64_t cap);
/* euclidean_search in a linearly transformed coordinate system
 * (LinearTransform / ScaleTransform, src/Transform.h; the search iterator's
 * m_dx = transform(p - x), src/Search.h:438-445): T is the row-major dim x dim
 * matrix of the transform, y = T dx evaluated as ((T_i0 dx_0 + T_i1 dx_1) +
 * T_i2 dx_2), and a particle is a neighbour iff !(((0 + y_0^2) + y_1^2) +
 * y_2^2 > r^2).  rowptr[nq+1] as abx_radius_query_csr; cols (may be NULL:
 * counts only) and dx[nnz*dim] (may be NULL) receive the neighbours and
 * their TRANSFORMED separations, as the reference's dx() returns them.  T
 * must be invertible. */
ABX_API int abx_radius_query_csr_transform(abx_particles *p, int64_t nq, const double *q,
                                           double r, const double *T, int64_t *rowptr,
                                           int32_t *cols, double *dx, int64_t cap);
/* Every pair of stored particles within r, once: the pairs a sweep over the
 * neighbouring buckets of the cell list visits (bucket_pair_iterator /
 * get_neighbouring_buckets, src/Search.h:498-764, plus the pairs inside each
 * bucket).  *npairs receives the count; pi, pj (both NULL: count only) and
 * dx[npairs*dim] (may be NULL) receive the pairs as storage indices with
 * pi < pj, in increasing pi, with dx = x_pj - (x_pi + image*L) of the image
 * the search accepted and !(|dx|^2 > r^2).  cap: capacity of pi/pj. */
ABX_API int abx_radius_pairs(abx_particles *p, double r, int64_t *npairs, int32_t *pi,
                             int32_t *pj, double *dx, int64_t cap);

/* k nearest neighbours of every stored particle among the stored particles
 * (itself included, FP64 distances with periodic images, ties by storage
 * index), k <= 64: idx[i*k + j] storage indices in increasing distance, d2
 * (optional) the squared distances.  No counterpart in the reference; used to
 * build the support of the learned sparse approximate inverse. */
ABX_API int abx_knn(abx_particles *p, int k, int32_t *idx, double *d2);

/* -------------------------------------------------------------- operators --
 * create_sparse_operator (src/Operators.h:478-515, KernelSparseConst
 * src/Kernels.h:754-776), create_dense_operator (src/Operators.h:312-318,
 * KernelDense src/Kernels.h:138-268).  The operator holds the particle sets by
 * reference (as the reference's kernels do, src/Kernels.h:133-135): they must
 * outlive it and not be re-searched while it is in use. */
ABX_API int abx_create_sparse_operator(abx_particles *rows, abx_particles *cols, double radius,
                               const abx_kernel *k, abx_operator **out);
ABX_API int abx_create_dense_operator(abx_particles *rows, abx_particles *cols, const abx_kernel *k,
                              abx_operator **out);
/* create_fmm_operator (src/Operators.h:401-407, KernelFMM src/Kernels.h:
 * 533-576): black-box Chebyshev FMM with `order` nodes per dimension on the
 * octree of p (abx_particles_init_octree; leaves of <= n_particles_in_leaf).
 * Kernels: ABX_K_LAPLACE, _GAUSSIAN, _COMPACT_GAUSSIAN (no cut-off),
 * _MULTIQUADRIC, _CONST.  ABX_PREC_FP64: every pass in FP64;
 * ABX_PREC_MIXED: M2L as 3xTF32 tensor-core GEMMs with FP32 accumulation and
 * P2P in FP32. */
ABX_API int abx_create_fmm_operator(abx_particles *p, const abx_kernel *k, int order,
                                    abx_operator **out);
/* create_h2_operator(particles, particles, order, kernel, eta)
 * (src/Operators.h:440-447; H2Matrix / make_h2_matrix, src/H2Matrix.h:46-110,
 * src/ParH2Matrix.h:564-570): the black-box Chebyshev H2 operator with a
 * runtime order and the admissibility parameter eta -- a box pair is far
 * (M2L) when its gap is at least (max diameter) / eta, eta = 1 being the
 * FMM's rule; a smaller eta keeps more pairs near and is more accurate.  The plan (tree traversal, M2L and child interpolation matrices, the
 * split-TF32 M2L images) is built once and reused by every K*b; the leaf
 * expansions and the near-field blocks are evaluated on the fly, which on the
 * GPU is cheaper than reading stored blocks from memory.  Matvec precision
 * and kernels as for abx_create_fmm_operator. */
ABX_API int abx_create_h2_operator(abx_particles *p, const abx_kernel *k, int order, double eta,
                                   abx_operator **out);
ABX_API int abx_fmm_stats(abx_operator *op, int64_t *m2l_pairs, int64_t *matrices,
                          int64_t *leaves, double *plan_seconds);
/* Limit of every device-side wait of the tensor-core M2L (its pipeline's
 * mbarriers), in seconds of the GPU's global timer (default 1 s, at most 60):
 * a wait that runs out makes the matvec return ABX_ERR_TIMEOUT after the
 * kernel has drained its copies and MMAs in flight and freed its tensor
 * memory, so the context stays usable.  drop_one_arrive = 1 is fault
 * injection for tests: the M2L producer withholds its first operand-ready
 * signal, so the MMA issuer's wait runs out (a barrier nothing arrives on);
 * 0 restores normal operation.  No counterpart in the reference, whose FMM
 * runs on the host. */
ABX_API int abx_fmm_set_wait_limit(abx_operator *op, double seconds, int drop_one_arrive);
ABX_API int abx_operator_destroy(abx_operator *op);
ABX_API int abx_operator_set_precision(abx_operator *op, int mode);
ABX_API int64_t abx_operator_rows(const abx_operator *op);
ABX_API int64_t abx_operator_cols(const abx_operator *op);
/* c = K*b (Eigen assignment semantics, generic_product_impl::scaleAndAddTo
 * src/detail/Operators.h:207-229 with alpha == 1 on a zeroed destination). */
ABX_API int abx_operator_matvec(abx_operator *op, const double *b, double *c);
/* Allocation-free variant of abx_operator_matvec for sparse operators (no
 * counterpart in the reference).  For callers that must not allocate device
 * memory while applying an operator -- code running under a device-memory
 * budget owned by another runtime, or a time-stepping loop that cannot pay
 * cudaMalloc/cudaFree's implicit device-wide synchronisation.  It calls no
 * cudaMalloc, cudaFree or allocating library routine: the per-call scratch
 * lives in one fixed 32 MiB device array inside the library, which every GPU
 * that loads the library holds until the process exits.
 *   - b and c must be device memory of the context's GPU (or managed memory);
 *     host vectors and other GPUs' memory are rejected (ABX_ERR_INVALID).
 *   - The scratch needed is 4 B (mixed precision) or 8 B (FP64) per column plus
 *     8 B per row, each rounded up to 256 B, plus 256 B; larger operators are
 *     rejected with ABX_ERR_CAPACITY (about 2.7M particles for a square mixed
 *     operator).
 *   - The operator must be current: if its particle sets were re-searched since
 *     it was built, the call fails with ABX_ERR_STATE instead of rebuilding.
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *   - All calls share the one array and it keeps the last call's contents, so
 *     calls that overlap on the GPU (other streams, other host threads) race;
 *     serialise them on one stream.
 */
ABX_API int abx_operator_matvec_noalloc(abx_operator *op, const double *b, double *c);
/* Pair work of the last matvec: candidate pairs tested and pairs accepted. */
ABX_API int abx_operator_last_stats(abx_operator *op, int64_t *candidates, int64_t *pairs);

/* ---------------------------------------------------------- solvers --
 * Preconditioners (x = M b) and restarted flexible GMRES. */
typedef struct abx_precond abx_precond;
/* SchwartzPreconditioner<LU> (src/Preconditioners.h:1121-1537): one domain per
 * non-empty octree leaf of the operator's particle set (rows == cols, set up
 * with abx_particles_init_octree); the block over the leaf's particles plus
 * those of every touching leaf is assembled with coeff (strict |dx| < r,
 * src/detail/Kernels.h:336-368) and LU-factorised in FP64.  precision
 * ABX_PREC_MIXED keeps FP32 copies of the factors for the apply.  Apply is
 * restricted additive Schwarz (src/Preconditioners.h:1477-1522). */
ABX_API int abx_precond_create_schwarz(abx_operator *op, int precision, abx_precond **out);
/* Sparse approximate inverse with k entries per row: x_i = sum_j vals[i*k+j] *
 * b[cols[i*k+j]] (the row form of CardinalFunctionsPreconditioner,
 * src/Preconditioners.h:1025-1103). */
ABX_API int abx_precond_create_spai(abx_context *ctx, int64_t n, int k, const int32_t *cols,
                                    const double *vals, abx_precond **out);
/* Exact FP64 least-squares approximate-inverse rows on a k-nearest-neighbour
 * support (k <= 32): CardinalFunctionsPreconditioner::factorize
 * (src/Preconditioners.h:1025-1082) with the support restricted to the k
 * nearest neighbours of each particle; column-pivoted Householder QR.  cols
 * and vals are n*k (storage indices / weights), usable with
 * abx_precond_create_spai; they are also the learned model's training
 * labels. */
ABX_API int abx_spai_exact_rows(abx_operator *op, int k, int32_t *cols, double *vals);
/* Schwarz block-solve rows on the k-nearest-neighbour domain: row i of
 * (A_SS)^{-1} restricted to i, i.e. the solve of the k x k local block
 * (SchwartzPreconditioner::factorize + _solve_impl, src/Preconditioners.h:
 * 1403-1522, with a one-particle restriction).  These are the learned
 * model's training labels. */
ABX_API int abx_spai_local_inverse_rows(abx_operator *op, int k, int32_t *cols, double *vals);
/* Features of the learned approximate inverse: feats[i][j*dim + d] =
 * eps * (x_{knn[i][j]} - x_i)_d (periodic minimum image), n*k*dim floats. */
ABX_API int abx_spai_features(abx_particles *p, const int32_t *knn, int k, double eps,
                              float *feats);
/* Learned sparse approximate inverse (no counterpart in the reference): k-NN
 * support, features as above, weights from the MLP (precision ABX_PREC_MIXED:
 * BF16 tensor-core inference; ABX_PREC_FP64: FP32 SIMT inference).  Rows
 * whose nearest other point has kernel value phi > exact_phi (phi(0) = 1 for
 * the Gaussian and Wendland kernels) are instead solved exactly as FP64
 * local-inverse rows (abx_spai_local_inverse_rows): next to a near-coincident
 * pair the inverse's weights grow like 1/(1 - phi) and cancel, which no
 * regression reproduces.  exact_phi >= 1: every row from the network. */
typedef struct abx_mlp abx_mlp;
ABX_API int abx_precond_create_learned(abx_operator *op, abx_mlp *mlp, double eps, int k,
                                       int precision, double exact_phi, abx_precond **out);
ABX_API int abx_precond_get_spai(abx_precond *pc, int32_t *cols, double *vals);
ABX_API int abx_precond_destroy(abx_precond *pc);
ABX_API int abx_precond_apply(abx_precond *pc, const double *b, double *x);
/* Schwarz: domains, largest domain, stored factor elements, set-up seconds.
 * Approximate inverses: ndomains = rows solved exactly, set-up seconds. */
ABX_API int abx_precond_stats(abx_precond *pc, int64_t *ndomains, int64_t *max_size,
                              int64_t *elements, double *setup_seconds);
/* Learned approximate inverse: device seconds of its set-up phases -- the
 * k-NN search, the features, the network's inference and the exact FP64 rows
 * next to close neighbours (CUDA events on the build stream; 0 for other
 * preconditioners).  No reference counterpart (the learned preconditioner is
 * new); any pointer may be NULL. */
ABX_API int abx_precond_setup_phases(abx_precond *pc, double *knn_s, double *features_s,
                                     double *infer_s, double *exact_s);
/* Solve A x = b (x holds the initial guess) with restarted, right-
 * preconditioned flexible GMRES(restart): CGS2 orthogonalisation and Givens
 * rotations in FP64.  At every restart the true residual b - A_check x is
 * recomputed with A_check (NULL: A); iteration stops when its norm relative to
 * |b| is <= tol or after max_iters inner iterations.  Passing a mixed-precision
 * A and an FP64 A_check gives iterative refinement with an FP64-checked
 * residual.  The reference's solvers are Eigen's (third party), used as
 * gmres.compute(W); gmres.solve(phi) in tests/rbf_interpolation.h:360-370. */
ABX_API int abx_gmres_solve(abx_operator *A, abx_operator *A_check, abx_precond *M,
                            const double *b, double *x, int restart, int max_iters, double tol,
                            int *iterations, double *rel_residual);

/* ---------------------------------------------------------------- MLP --
 * The learned preconditioner's model (no counterpart in the reference):
 * in_dim -> nhidden x hidden (SiLU) -> out_dim, FP32 parameters, trained with
 * the library's own forward/backward/Adam kernels on normalised targets
 * ((y - out_shift) / out_scale), inference in BF16 on the tensor cores. */
ABX_API int abx_mlp_create(abx_context *ctx, int in_dim, int hidden, int nhidden, int out_dim,
                           uint64_t seed, abx_mlp **out);
ABX_API int abx_mlp_destroy(abx_mlp *mlp);
ABX_API int64_t abx_mlp_num_params(const abx_mlp *mlp);
ABX_API int abx_mlp_set_normalization(abx_mlp *mlp, float in_scale, const float *out_scale,
                                      const float *out_shift);
/* Output transform applied after denormalisation at inference: kind 0 none,
 * kind 1 y -> c * sinh(y) (for targets trained as asinh(w / c)). */
ABX_API int abx_mlp_set_output_transform(abx_mlp *mlp, int kind, float c);
ABX_API int abx_mlp_get_params(abx_mlp *mlp, float *params);
ABX_API int abx_mlp_set_params(abx_mlp *mlp, const float *params);
/* Training loss of abx_mlp_gradients / abx_mlp_train_step.
 *   ABX_LOSS_MSE (default): mean squared error on normalised targets y.
 *   ABX_LOSS_SPAI_RESIDUAL: the approximate-inverse residual of each row,
 *     mean_i |A_i m_i - e_0|^2, with m_i the denormalised output (k = out_dim
 *     weights, output transform 0) and A_i the k x k kernel matrix of the
 *     row's support read from its features x_i = (f_0 .. f_{k-1}), f_a in
 *     R^dim (in_dim = k*dim, f_0 the row's own point): A_ab = kern(f_b - f_a)
 *     when |f_b - f_a| < cutoff, else 0.  e_0 selects the row's own point.
 *     Targets are not used (y may be NULL).  Errors in directions the
 *     operator barely sees cost little, which a weight MSE cannot express.
 * No counterpart in the reference. */
#define ABX_LOSS_MSE 0
#define ABX_LOSS_SPAI_RESIDUAL 1
ABX_API int abx_mlp_set_loss(abx_mlp *mlp, int kind, int dim, const abx_kernel *k, double cutoff);
/* Loss and its gradient w.r.t. the flat parameters for one batch, without
 * updating. */
ABX_API int abx_mlp_gradients(abx_mlp *mlp, const float *x, const float *y, int64_t batch,
                              float *grads, float *loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on one batch. */
ABX_API int abx_mlp_train_step(abx_mlp *mlp, const float *x, const float *y, int64_t batch,
                               float lr, float *loss);
/* y = model(x) (denormalised); precision ABX_PREC_MIXED = BF16 tensor cores. */
ABX_API int abx_mlp_forward(abx_mlp *mlp, const float *x, int64_t n, float *y, int precision);
ABX_API int abx_mlp_save(abx_mlp *mlp, const char *path);
ABX_API int abx_mlp_load(abx_context *ctx, const char *path, abx_mlp **out);

/* Learned-then-fallback solve: GMRES with M_learned for at most
 * learned_max_iters iterations; if that does not reach tol, the restricted
 * additive Schwarz preconditioner of A_fallback (an FP64 sparse operator on
 * an octree particle set) is built and GMRES continues from the current x.
 * *used_fallback reports which preconditioner finished the solve. */
ABX_API int abx_gmres_solve_fallback(abx_operator *A, abx_operator *A_check, abx_precond *M_learned,
                                     abx_operator *A_fallback, const double *b, double *x,
                                     int restart, int learned_max_iters, int max_iters,
                                     double tol, int *iterations, double *rel_residual,
                                     int *used_fallback);

/* ------------------------------------------------------------ diagnostics --
 * Measured FP32 throughput of this GPU (no counterpart in the reference): the
 * denominator of the pair kernels' compute roofline.  8 CTAs x 256 threads per
 * SM run independent FMA chains, `iters` steps of 8 chains per thread, scalar
 * FFMA (packed = 0) or packed FP32x2 FFMA2 (packed = 1); best of three timed
 * launches after a warm-up, CUDA events on the context's stream.  *tflops
 * counts an FMA as 2 FLOP. */
ABX_API int abx_probe_fp32_peak(abx_context *ctx, int packed, int iters, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* ABX_H_ */
