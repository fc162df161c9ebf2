"""Full-size checks on the sparse-operator benchmark workload itself
(``bench.make_workload()``: N = 4,194,304, 16-Gaussian mixture + 20% uniform,
periodic unit box, r = 0.02, Wendland C2, b ~ N(0,1)).

Against the oracle (the reference's algorithm restated, OpenMP on the host):

* the cell order equals the oracle's stable (bucket key, insertion) order;
* all 4,194,304 radius counts equal the oracle's (src/Search.h:438-465);
* neighbour sets are bit-exact on 10,000 sampled rows plus the 200 densest
  rows (the cluster cores, ~9,000 neighbours each);
* the FP64-mode matvec is within 1e-12 (relative L2) of the oracle's FP64
  matvec (src/Kernels.h:720-751) on 1,048,576 rows, a contiguous quarter of
  the storage order plus the densest rows; the mixed mode within 2e-6.

Size-independent properties on top:

* sortedness of the cell list; rebuilding is idempotent;
* a checksum of checksums: K * 1 with the constant kernel (value 1) is, row
  by row, the neighbour count -- in FP64 and in mixed precision (FP32 blocks of
  ones are exact) it must equal the radius-count kernel's counts exactly;
* linearity of the mixed Wendland operator; symmetry of the FP64 one
  (b1 . K b2 = b2 . K b1, the kernel being symmetric and rows == cols).
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import bench
import oracle

pytestmark = pytest.mark.gpu

N, R = bench.N_PARTICLES, bench.RADIUS
LO, HI, PER = [0.0] * 3, [1.0] * 3, [True] * 3


@pytest.fixture(scope="module")
def cfg2():
    pos, b_by_id = bench.make_workload()
    p = ab.Particles(3).set(pos)
    p.init_neighbour_search(LO, HI, PER, 10.0)
    cl = oracle.celllist_build(pos, LO, HI, PER, 10.0)
    counts = ab.radius_count(p, p.positions, R)
    return p, cl, b_by_id, counts


def test_cell_order_matches_oracle(cfg2):
    p, cl, _, _ = cfg2
    assert np.array_equal(p.ids, cl.perm)
    assert np.array_equal(p.positions, cl.pos)
    bb, be, keys = p.buckets()
    assert np.array_equal(keys, cl.keys)
    assert np.array_equal(bb, cl.begin) and np.array_equal(be, cl.end)


def test_all_counts_match_oracle(cfg2):
    p, cl, _, counts = cfg2
    ref = oracle.radius_count(cl, cl.pos, R)
    assert counts.shape == (N,)
    bad = np.nonzero(counts != ref)[0]
    assert bad.size == 0, f"{bad.size} rows differ, first {bad[:5]}"


def _sample_rows(counts, n_random, n_dense, seed):
    rng = np.random.default_rng(seed)
    rand = rng.choice(N, n_random, replace=False)
    dense = np.argsort(counts, kind="stable")[-n_dense:]
    return np.unique(np.concatenate([rand, dense]))


def test_neighbour_sets_sampled_and_densest(cfg2):
    p, cl, _, counts = cfg2
    rows = _sample_rows(counts, 10_000, 200, seed=31)
    q = cl.pos[rows]
    rowptr, cols = ab.radius_query_csr(p, q, R)
    orp, ocols, _ = oracle.radius_lists(cl, q, R)
    assert np.array_equal(rowptr, orp)
    assert counts[rows].max() > 5000  # the densest cluster rows are included
    for i in range(len(rows)):
        a = np.sort(cols[rowptr[i]:rowptr[i + 1]])
        b = np.sort(ocols[orp[i]:orp[i + 1]])
        assert np.array_equal(a, b), f"row {rows[i]}"


def test_matvec_matches_oracle_on_a_million_rows(cfg2):
    p, cl, b_by_id, counts = cfg2
    b = np.ascontiguousarray(b_by_id[p.ids])
    quarter = np.arange(N // 4, N // 2)
    rows = np.unique(np.concatenate([quarter, np.argsort(counts, kind="stable")[-2000:]]))
    assert rows.size >= 1_048_576
    kern = ab.Kernel.make(ab.K_WENDLAND_C2, 1.0 / R)
    ref = oracle.sparse_matvec(cl, cl.pos[rows], R, ab.K_WENDLAND_C2, [1.0 / R], b)
    K64 = ab.create_sparse_operator(p, p, R, kern, ab.PREC_FP64)
    c64 = (K64 * b)[rows]
    del K64
    e64 = np.linalg.norm(c64 - ref) / np.linalg.norm(ref)
    assert e64 <= 1e-12, e64
    K32 = ab.create_sparse_operator(p, p, R, kern, ab.PREC_MIXED)
    c32 = (K32 * b)[rows]
    e32 = np.linalg.norm(c32 - ref) / np.linalg.norm(ref)
    assert e32 <= 2e-6, e32


def test_cell_list_sorted_and_idempotent(cfg2):
    p = cfg2[0]
    bb, be, keys = p.buckets()
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    assert np.all(be >= bb) and int((be - bb).astype(np.int64).sum()) == N
    nz = be > bb
    assert np.all(keys[bb[nz]] == np.nonzero(nz)[0])
    ids = p.ids
    p.init_neighbour_search(LO, HI, PER, 10.0)
    assert np.array_equal(p.ids, ids)


def test_constant_kernel_matvec_equals_counts(cfg2):
    p, _, _, counts = cfg2
    assert counts.min() >= 1  # every particle is its own neighbour
    ones = np.ones(N)
    kern = ab.Kernel.make(ab.K_CONST, 1.0)
    for prec in (ab.PREC_MIXED, ab.PREC_FP64):
        K = ab.create_sparse_operator(p, p, R, kern, prec)
        c = K * ones
        assert np.array_equal(c, counts.astype(np.float64)), prec
        del K


def test_linearity_and_symmetry(cfg2):
    p = cfg2[0]
    rng = np.random.default_rng(7)
    b1, b2 = rng.standard_normal(N), rng.standard_normal(N)
    kern = ab.Kernel.make(ab.K_WENDLAND_C2, 1.0 / R)
    K32 = ab.create_sparse_operator(p, p, R, kern, ab.PREC_MIXED)
    k1, k2 = K32 * b1, K32 * b2
    k12 = K32 * (2.0 * b1 + b2)
    assert np.linalg.norm(k12 - (2.0 * k1 + k2)) / np.linalg.norm(k12) < 2e-6
    del K32
    K64 = ab.create_sparse_operator(p, p, R, kern, ab.PREC_FP64)
    a, b = b1 @ (K64 * b2), b2 @ (K64 * b1)
    assert abs(a - b) <= 1e-10 * (abs(a) + abs(b))
