"""Oracle neighbour search: the cell walk of neighborhood_green.comp with the
canonical integer predicate must equal an O(n^2) brute force, including variable
ranges, particles outside the grid bounds, and the empty case."""
import numpy as np
import pytest

from apbf_gb300 import scenes


def _random_state(n, seed, spread=20.0, kw_lo=4.0, kw_hi=4.0):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-spread * 0.1, spread, size=(n, 3))
    st = scenes.make_state(pos)
    st["kernel_width"] = rng.uniform(kw_lo, kw_hi, size=n).astype(np.float32)
    return st


@pytest.mark.parametrize("seed,kw_hi,L", [(0, 4.0, 3), (1, 9.0, 4), (2, 2.5, 5)])
def test_green_equals_brute_force(orc, seed, kw_hi, L):
    st = _random_state(700, seed, kw_lo=2.0, kw_hi=kw_hi)
    fs = orc.FluidState(st)
    perm, keys, tot = orc.neighborhood_green(fs, 1.0, (0.0, 0.0, 0.0), (16.0, 16.0, 16.0), L, 1 << 20)
    # state was reordered by the sort: brute force on the reordered state
    s2 = fs.state()
    brute = orc.neighbors_brute(s2["position"], s2["kernel_width"], 1.0)
    rows = fs.rows()
    assert sum(len(r) for r in rows) == tot
    for i in range(fs.n):
        assert np.array_equal(rows[i], brute[i]), i
    # the permutation is the stable sort of the keys of the original order
    k0 = orc.position_keys(st["position"], (0.0, 0.0, 0.0), (16.0, 16.0, 16.0), L)
    assert np.array_equal(perm, np.argsort(k0, kind="stable").astype(np.uint32))
    assert np.array_equal(keys, k0[perm])
    assert np.array_equal(s2["position"], st["position"][perm])


def test_micro_case_like_disabled_reference_test(orc):
    # test.cpp:561-565 (disabled there): particles at (0,0,0), (1,0,0), (0,1,0), ranges 1, 1, 2
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float64)
    st = scenes.make_state(pos)
    st["kernel_width"] = np.array([1.0, 1.0, 2.0], np.float32)
    rows = orc.neighbors_brute(st["position"], st["kernel_width"], 1.0)
    assert [r.tolist() for r in rows] == [[1, 2], [0], [0, 1]]
    fs = orc.FluidState(st)
    orc.neighborhood_green(fs, 1.0, (-10.0, -10.0, -10.0), (10.0, 10.0, 10.0), 6, 64)
    s2 = fs.state()
    brute = orc.neighbors_brute(s2["position"], s2["kernel_width"], 1.0)
    assert [r.tolist() for r in fs.rows()] == [r.tolist() for r in brute]


def test_empty_and_single(orc):
    for n in (0, 1):
        st = _random_state(n, 0)
        fs = orc.FluidState(st, cap=4)
        perm, keys, tot = orc.neighborhood_green(fs, 1.0, (0.0, 0.0, 0.0), (16.0, 16.0, 16.0), 3, 16)
        assert tot == 0 and perm.size == n


def test_cell_clamp(orc):
    lo, hi = 0, 16 * 262144
    assert orc.lib().or_cell_coord(-5, lo, hi, 4) == 0
    assert orc.lib().or_cell_coord(hi + 7, lo, hi, 4) == 15
    assert orc.lib().or_cell_coord(hi - 1, lo, hi, 4) == 15
    assert orc.lib().or_cell_coord(262144, lo, hi, 4) == 1


def test_range_fixed_is_floor(orc):
    assert orc.lib().or_range_fixed(4.0, 1.0) == 4 * 262144
    assert orc.lib().or_range_fixed(4.0, 1.5) == 6 * 262144
    assert orc.lib().or_range_fixed(float("nan"), 1.0) == -1
