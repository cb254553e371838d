"""Oracle binary-search neighbour search (neighborhood_binary_search.cpp:22-75,
neighborhood_binary_search.comp, calculate_position_code.comp): the 96-bit code
against a bit-by-bit interleave, the sort order against a stable lexicographic
sort, the rows against an O(n^2) brute force as sets and against a pure-Python walk
of the 27 cells for their order, across the sign boundary of the coordinates and at
the largest cell level."""
import numpy as np
import pytest

from apbf_gb300 import scenes


def _code_py(p):
    c = 0
    for b in range(32):
        for a in range(3):
            if (int(p[a]) & 0xFFFFFFFF) >> b & 1:
                c |= 1 << (3 * b + a)
    return c


def _words(c):
    return [(c >> (32 * w)) & 0xFFFFFFFF for w in range(3)]


def test_position_code_interleave(orc):
    rng = np.random.default_rng(0)
    pos = rng.integers(-(2 ** 31), 2 ** 31, size=(300, 4), dtype=np.int64).astype(np.int32)
    pos[:4, :3] = [[0, 0, 0], [-1, -1, -1], [2 ** 31 - 1, -(2 ** 31), 1], [1, 2, 4]]
    got = orc.position_codes(pos)
    for i in range(pos.shape[0]):
        assert got[i].tolist() == _words(_code_py(pos[i, :3])), i
    # (1, 2, 4): x bit 0 -> code bit 0, y bit 1 -> code bit 4, z bit 2 -> code bit 8
    assert got[3].tolist() == [(1 << 0) | (1 << 4) | (1 << 8), 0, 0]


def _state(n, seed, lo, hi, kw_lo, kw_hi, dups=0):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(lo, hi, size=(n, 3))
    if dups:
        pos[-dups:] = pos[:dups]  # equal positions: equal codes
    st = scenes.make_state(pos)
    st["kernel_width"] = rng.uniform(kw_lo, kw_hi, size=n).astype(np.float32)
    return st


def _rows_py(pos4, codes, kw, scale, orc):
    """The 27-cell walk in plain Python (small n)."""
    n = pos4.shape[0]
    full = [int(c[0]) | int(c[1]) << 32 | int(c[2]) << 64 for c in codes]
    rows = []
    for i in range(n):
        R = int(orc.lib().or_range_fixed(float(kw[i]), scale))
        k = 0
        while (1 << k) < R:
            k += 1
        offs = (-1, 0) if k == 31 else (-1, 0, 1)
        row = []
        for dz in offs:
            for dy in offs:
                for dx in offs:
                    corner = [((((int(pos4[i, a]) & 0xFFFFFFFF) >> k) + d) << k) & 0xFFFFFFFF
                              for a, d in enumerate((dx, dy, dz))]
                    first = _code_py(corner)
                    last = first | ((1 << (3 * k)) - 1)
                    for j in range(n):
                        if j == i or not first <= full[j] <= last:
                            continue
                        d = pos4[j, :3].astype(np.int64) - pos4[i, :3].astype(np.int64)
                        if np.all(np.abs(d) <= R) and int(np.sum(d * d)) <= R * R:
                            row.append(j)
        rows.append(row)
    return rows


@pytest.mark.parametrize("seed,lo,hi,kw_lo,kw_hi,dups", [
    (1, 0.0, 20.0, 2.0, 4.0, 0),
    (2, -10.0, 10.0, 1.0, 6.0, 20),   # across the sign boundary of every axis
    (3, -3000.0, 3000.0, 3000.0, 9000.0, 0),  # levels up to 31: two cells per axis
])
def test_binary_search_rows(orc, seed, lo, hi, kw_lo, kw_hi, dups):
    st = _state(260, seed, lo, hi, kw_lo, kw_hi, dups)
    fs = orc.FluidState(st)
    perm, codes, tot = orc.neighborhood_binary_search(fs, 1.0, 1 << 20)
    s2 = fs.state()
    # the permutation: stable sort by the 96-bit code of the original order
    c0 = orc.position_codes(st["position"])
    order = np.lexsort((np.arange(c0.shape[0]), c0[:, 0], c0[:, 1], c0[:, 2]))
    assert np.array_equal(perm, order.astype(np.uint32))
    assert np.array_equal(codes, c0[perm])
    assert np.array_equal(s2["position"], st["position"][perm])
    # rows: the brute-force neighbours, each once, in the 27-cell walk's order
    rows = fs.rows()
    assert sum(len(r) for r in rows) == tot
    brute = orc.neighbors_brute(s2["position"], s2["kernel_width"], 1.0)
    for i in range(fs.n):
        assert np.array_equal(np.sort(rows[i]), brute[i]), i
    walk = _rows_py(s2["position"], codes, s2["kernel_width"], 1.0, orc)
    for i in range(fs.n):
        assert rows[i].tolist() == walk[i], i
    if seed == 3:
        assert max(len(r) for r in rows) == fs.n - 1  # the whole set is in range


def test_binary_search_empty_and_single(orc):
    for n in (0, 1):
        st = _state(n, 0, 0.0, 10.0, 4.0, 4.0)
        fs = orc.FluidState(st, cap=4)
        perm, codes, tot = orc.neighborhood_binary_search(fs, 1.0, 16)
        assert tot == 0 and perm.size == n


def test_substep_with_binary_search_equals_green_as_sets(orc):
    """A whole oracle substep with either search: the same particles (as a set of
    states) -- the Jacobi sums are order-free -- when no step depends on the id."""
    spec = scenes.dam_break(n_side=8)
    out = []
    for method in (1, 3):
        fs = orc.FluidState(spec.state)
        s = orc.settings_from(dict(height_kernel_id=1, gradient_kernel_id=1, basic_pbf=1, solver_iterations=3,
                                   boundariness_calculation_method=2, update_boundariness=1,
                                   boundariness_adaption_speed=0.5, boundariness_self_grad_length_factor=2.0,
                                   boundariness_underpressure_factor=4.0))
        sc = orc.make_scene(s, spec.grid_min, spec.grid_max, spec.log2res, spec.acceleration, search_method=method)
        no_boxes = (np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32))
        for _ in range(3):
            orc.substep(fs, sc, no_boxes, np.float32(spec.dt), 1 << 20)
        o = fs.state()
        key = np.lexsort(o["position"][:, :3].T[::-1])
        out.append({k: v[key] for k, v in o.items()})
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
