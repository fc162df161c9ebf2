"""GPU CellListOrdered build vs the oracle: bit-exact order, keys and buckets.

The stable order (bucket key, insertion index) is the reference's Thrust
backend order (src/detail/Algorithms.h:193-196); buckets follow
lower_bound/upper_bound (src/CellListOrdered.h:231-239).
"""
import numpy as np
import pytest

import aboria_gb300 as ab
import oracle
import workloads

pytestmark = pytest.mark.gpu


def check_build(pos, lo, hi, periodic, n_leaf=10.0):
    dim = pos.shape[1]
    p = ab.Particles(dim).set(pos)
    p.init_neighbour_search(lo, hi, periodic, n_leaf)
    cl = oracle.celllist_build(pos, lo, hi, periodic, n_leaf, stable=True)
    size, side, nc = p.grid()
    assert list(size) == list(cl.size)
    assert np.array_equal(side, cl.side)
    assert len(p) == cl.n
    assert np.array_equal(p.ids, cl.perm)
    assert np.array_equal(p.positions, cl.pos)  # bit-exact, incl. periodic wrap
    bb, be, keys = p.buckets()
    assert np.array_equal(keys, cl.keys)
    assert np.array_equal(bb, cl.begin) and np.array_equal(be, cl.end)
    return p, cl


def test_cfg1_uniform_nonperiodic():
    check_build(workloads.uniform(100000, 3, seed=1), [0] * 3, [1] * 3, [False] * 3)


def test_mixture_periodic_wrap():
    pos = workloads.gaussian_mixture(200000, 3, seed=2, periodic=False)  # unwrapped: needs wrap
    check_build(pos, [0] * 3, [1] * 3, [True] * 3)


def test_deletion_of_outside_and_nonfinite():
    pos = workloads.uniform(50000, 3, lo=-0.1, hi=1.1, seed=3)
    pos[::97, 1] = np.nan
    pos[::101, 2] = np.inf
    p, cl = check_build(pos, [0] * 3, [1] * 3, [False] * 3)
    assert len(p) < 50000


@pytest.mark.parametrize("dim", [1, 2])
def test_low_dimensions(dim):
    check_build(workloads.uniform(30000, dim, seed=4 + dim), [0] * dim, [1] * dim, [True] * dim)


@pytest.mark.parametrize("n_leaf", [1.0, 3.5, 100.0, 1e6])
def test_leaf_sizes(n_leaf):
    check_build(workloads.float_uniform(5000, 3, seed=5), [-1] * 3, [1] * 3, [False] * 3, n_leaf)


def test_tiny_and_empty_sets():
    check_build(np.array([[0.5, 0.5, 0.5]]), [0] * 3, [1] * 3, [False] * 3)
    check_build(np.zeros((0, 3)), [0] * 3, [1] * 3, [False] * 3)
    # everything deleted
    p = ab.Particles(3).set(np.full((10, 3), 2.0))
    p.init_neighbour_search([0] * 3, [1] * 3, [False] * 3)
    assert len(p) == 0


def test_anisotropic_domain_and_duplicates():
    rng = np.random.default_rng(6)
    pos = rng.uniform(0, 1, size=(20000, 3)) * [4.0, 1.0, 0.25] + [-2.0, 0.0, 5.0]
    pos[1000:2000] = pos[0]  # many identical points in one bucket
    check_build(pos, [-2.0, 0.0, 5.0], [2.0, 1.0, 5.25], [True, False, True])


def test_rebuild_after_moving_particles():
    pos = workloads.uniform(40000, 3, seed=7)
    p = ab.Particles(3).set(pos)
    p.init_neighbour_search([0] * 3, [1] * 3, [True] * 3)
    ids_before = p.ids
    moved = p.positions + 0.3  # in the current (cell) storage order
    p.set_positions(moved)
    p.update_positions()
    cl = oracle.celllist_build(moved, [0] * 3, [1] * 3, [True] * 3)
    assert np.array_equal(p.ids, ids_before[cl.perm])
    assert np.array_equal(p.positions, cl.pos)


@pytest.mark.parametrize("frac_deleted,keeps_grid", [(0.3, True), (0.6, False)])
def test_grid_hysteresis_after_deletion(frac_deleted, keeps_grid):
    """set_domain_impl recomputes the grid only when the alive count leaves
    [0.5, 2] x the count it was computed with (src/CellListOrdered.h:133-136):
    deleting 30% keeps the old grid, deleting 60% recomputes it.  The rebuilt
    order, keys and buckets must equal the oracle's with the same rule."""
    n = 100000
    pos = workloads.uniform(n, 3, seed=8)
    p = ab.Particles(3).set(pos)
    p.init_neighbour_search([0] * 3, [1] * 3, [False] * 3)
    size0 = p.grid()[0].copy()
    ids_before = p.ids
    moved = p.positions
    kill = np.random.default_rng(9).random(n) < frac_deleted
    moved[kill] = 2.0  # outside the non-periodic domain: deleted
    p.set_positions(moved)
    p.update_positions()
    cl = oracle.celllist_build(moved, [0] * 3, [1] * 3, [False] * 3, prev_grid_n=n)
    size, side, _ = p.grid()
    assert list(size) == list(cl.size)
    assert np.array_equal(side, cl.side)
    assert np.array_equal(size, size0) == keeps_grid
    assert len(p) == cl.n == n - int(kill.sum())
    assert np.array_equal(p.ids, ids_before[cl.perm])
    assert np.array_equal(p.positions, cl.pos)
    bb, be, keys = p.buckets()
    assert np.array_equal(keys, cl.keys)
    assert np.array_equal(bb, cl.begin) and np.array_equal(be, cl.end)
    counts = ab.radius_count(p, p.positions, 0.05)
    assert np.array_equal(counts, oracle.radius_count(cl, cl.pos, 0.05))


def test_push_back_erase_and_find_by_id():
    """push_back / erase on a searchable set update the search structure at
    once (src/Particles.h:264-311, 361-389): the new order equals the oracle's
    build over the storage order before the update plus the new particles,
    with the grid kept within the 2x band (src/CellListOrdered.h:133-136).
    find-by-id (src/NeighbourSearchBase.h:276-321) maps ids to storage
    positions, -1 for erased ids."""
    n = 60000
    rng = np.random.default_rng(20)
    p = ab.Particles(3).set(workloads.uniform(n, 3, seed=21))
    p.init_neighbour_search([0] * 3, [1] * 3, [True] * 3)
    before_pos, before_ids = p.positions, p.ids
    extra = rng.uniform(-0.2, 1.2, size=(5000, 3))  # outside coordinates wrap
    new_ids = p.push_back(extra)
    assert np.array_equal(new_ids, np.arange(n, n + 5000))
    allpos = np.concatenate([before_pos, extra])
    allids = np.concatenate([before_ids, new_ids])
    cl = oracle.celllist_build(allpos, [0] * 3, [1] * 3, [True] * 3, prev_grid_n=n)
    assert np.array_equal(p.ids, allids[cl.perm])
    assert np.array_equal(p.positions, cl.pos)
    bb, be, keys = p.buckets()
    assert np.array_equal(keys, cl.keys) and np.array_equal(bb, cl.begin)
    # erase a storage range
    pos2, ids2 = p.positions, p.ids
    p.erase(1000, 4000)
    keep = np.r_[0:1000, 4000:len(ids2)]
    cl2 = oracle.celllist_build(pos2[keep], [0] * 3, [1] * 3, [True] * 3, prev_grid_n=n)
    assert np.array_equal(p.ids, ids2[keep][cl2.perm])
    assert np.array_equal(p.positions, cl2.pos)
    # find by id: present ids map to their storage index, erased ones to -1
    q = np.concatenate([rng.choice(p.ids, 3000), ids2[1000:1100], [-5, 10 ** 12]])
    idx = p.find_ids(q)
    ids_now = p.ids
    assert np.all(ids_now[idx[:3000]] == q[:3000])
    assert np.all(idx[3000:] == -1)
    counts = ab.radius_count(p, p.positions, 0.05)
    assert np.array_equal(counts, oracle.radius_count(cl2, cl2.pos, 0.05))


def test_erase_without_search_keeps_order():
    p = ab.Particles(2).set(workloads.uniform(100, 2, seed=22))
    ids = p.ids
    p.erase(10, 20)
    assert np.array_equal(p.ids, np.r_[ids[:10], ids[20:]])
    assert np.array_equal(p.find_ids(ids[:30]), np.r_[np.arange(10), [-1] * 10, np.arange(10, 20)])
