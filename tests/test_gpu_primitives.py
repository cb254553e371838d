"""GPU parity of the parallel primitives (algorithms::sort / prefix_sum) through the
C ABI: the reference's known answers (source/test.cpp) and seeded large cases,
bit-exact against the oracle / numpy."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(cuda):
    from apbf_gb300.api import Context

    c = Context(particle_capacity=600_000, max_neighbors=4, max_log2res=4)
    yield c
    c.close()


def _dev(a, dt=torch.int32):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


def _sort(ctx, keys, vals, ub=0xFFFFFFFF, max_count=None):
    from apbf_gb300.api import algorithms

    n = keys.size
    mc = max_count or max(n, 1)
    k = torch.zeros(mc, dtype=torch.int32, device="cuda")
    v = torch.zeros(mc, dtype=torch.int32, device="cuda")
    k[:n] = _dev(keys.astype(np.uint32))
    v[:n] = _dev(vals.astype(np.uint32))
    ok = torch.zeros_like(k)
    ov = torch.zeros_like(v)
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    algorithms.sort(ctx, k, v, cnt, mc, ok, ov, ub)
    ctx.check_status()
    return ok[:n].cpu().numpy().view(np.uint32), ov[:n].cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("name,cap", [("sort", None), ("sort_small_values", None),
                                      ("sort_few_values_in_long_buffer", 10000)])
def test_sort_known_answers(ctx, golden, name, cap):  # test.cpp:284-305, 343-364, 402-425
    v = golden[name]["vectors"]
    k, i = _sort(ctx, np.array(v["listData"], np.uint64), np.array(v["indexData"]), max_count=cap)
    assert k.tolist() == v["expectedResult"]
    assert i.tolist() == v["expectedIndexResult"]


@pytest.mark.parametrize("n,mask,ub", [(512 * 512 + 123, 0xFFFFFFFF, 0xFFFFFFFF), (512 * 512 + 1000, 15, 15),
                                       (100_000, (1 << 21) - 1, 1 << 21), (5000, (1 << 15) - 1, 1 << 15),
                                       (1, 7, 7), (4097, 255, 255)])
def test_sort_large_stable(ctx, orc, n, mask, ub):  # test.cpp:307-341, 366-400
    rng = np.random.default_rng(n)
    keys = (rng.integers(0, 1 << 32, size=n, dtype=np.uint64) & mask).astype(np.uint32)
    if n > 1000:
        keys[: n // 3] = np.sort(keys[: n // 3])  # partly presorted, like Morton keys between substeps
    vals = np.arange(n, dtype=np.uint32)
    k, i = _sort(ctx, keys, vals, ub)
    ok, oi = orc.sort_pairs(keys, vals)
    assert np.array_equal(k, ok)
    assert np.array_equal(i, oi)


def test_sort_respects_upper_bound_digits(ctx, orc):
    # keys above the upper bound: only the 4-bit digits below bitlen(ub) are sorted (algorithms.cpp:73)
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 1 << 20, size=3000, dtype=np.uint64).astype(np.uint32)
    k, i = _sort(ctx, keys, np.arange(3000, dtype=np.uint32), ub=255)
    low = keys & 255
    assert np.array_equal(i, np.argsort(low, kind="stable").astype(np.uint32))


def test_sort_empty(ctx):
    k, i = _sort(ctx, np.zeros(0, np.uint32), np.zeros(0, np.uint32), max_count=16)
    assert k.size == 0


@pytest.mark.parametrize("name", ["prefix_sum", "short_prefix_sum_in_long_buffer"])
def test_prefix_sum_known_answers(ctx, golden, name):  # test.cpp:186-197, 269-282
    from apbf_gb300.api import algorithms

    v = golden[name]["vectors"]
    mc = 10000 if "long" in name else len(v["listData"])
    t = torch.zeros(mc, dtype=torch.int32, device="cuda")
    t[: len(v["listData"])] = _dev(np.array(v["listData"], np.uint32))
    algorithms.prefix_sum(ctx, t, torch.tensor([len(v["listData"])], dtype=torch.int32, device="cuda"), mc)
    ctx.check_status()
    assert t[: len(v["listData"])].cpu().numpy().view(np.uint32).tolist() == v["expectedResult"]


@pytest.mark.parametrize("n,bits", [(1000, 2), (512 * 512 + 1000, 1), (500_000, 12)])
def test_prefix_sum_large(ctx, orc, n, bits):  # test.cpp:199-267
    from apbf_gb300.api import algorithms

    rng = np.random.default_rng(n)
    v = rng.integers(0, 1 << bits, size=n, dtype=np.uint32)
    t = _dev(v)
    algorithms.prefix_sum(ctx, t, torch.tensor([n], dtype=torch.int32, device="cuda"), n)
    ctx.check_status()
    assert np.array_equal(t.cpu().numpy().view(np.uint32), orc.prefix_sum(v))


@pytest.mark.parametrize("bits", [6, 7, 8])
def test_sort_digit_widths_give_the_same_order(ctx, orc, bits):
    """The tuned digit width (6, 7 or 8 bits per pass) changes the passes, not the
    stable order."""
    rng = np.random.default_rng(bits)
    n = 300_001
    keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 2] &= 0xFFF  # many equal keys: stability matters
    vals = np.arange(n, dtype=np.uint32)
    ctx.set_tuning(sort_digit_bits=bits)
    try:
        k, i = _sort(ctx, keys, vals)
        k21, i21 = _sort(ctx, keys & ((1 << 21) - 1), vals, ub=1 << 21)
    finally:
        ctx.set_tuning(sort_digit_bits=0)
    ok, oi = orc.sort_pairs(keys, vals)
    assert np.array_equal(k, ok) and np.array_equal(i, oi)
    ok21, oi21 = orc.sort_pairs(keys & ((1 << 21) - 1), vals)
    assert np.array_equal(k21, ok21) and np.array_equal(i21, oi21)
