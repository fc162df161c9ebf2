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
