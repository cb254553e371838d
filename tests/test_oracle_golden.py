"""Pins the oracle's primitives and list edits to the reference's own known-answer
tests (source/test.cpp), plus seeded large cases against independent numpy
implementations of the same semantics (stable sort, inclusive scan)."""
import numpy as np
import pytest


def test_prefix_sum_known_answers(orc, golden):
    for name in ("prefix_sum", "short_prefix_sum_in_long_buffer"):  # test.cpp:186-197, 269-282
        v = golden[name]["vectors"]
        assert orc.prefix_sum(np.array(v["listData"])).tolist() == v["expectedResult"]


@pytest.mark.parametrize("n,bits", [(1000, 2), (512 * 512 + 1000, 1)])
def test_prefix_sum_long(orc, n, bits):
    # test.cpp:199-267 use MSVC rand() after srand(0); same shapes, own seeded PRNG
    rng = np.random.default_rng(0)
    v = rng.integers(0, 1 << bits, size=n, dtype=np.uint32)
    assert np.array_equal(orc.prefix_sum(v), np.cumsum(v, dtype=np.uint64).astype(np.uint32))


def test_prefix_sum_empty(orc):
    assert orc.prefix_sum(np.zeros(0, np.uint32)).size == 0


@pytest.mark.parametrize("name", ["sort", "sort_small_values", "sort_few_values_in_long_buffer"])
def test_sort_known_answers(orc, golden, name):  # test.cpp:284-305, 343-364, 402-425
    v = golden[name]["vectors"]
    k, i = orc.sort_pairs(np.array(v["listData"]), np.array(v["indexData"]))
    assert k.tolist() == v["expectedResult"]
    assert i.tolist() == v["expectedIndexResult"]


@pytest.mark.parametrize("n,mask", [(512 * 512 + 123, 0xFFFFFFFF), (512 * 512 + 1000, 15), (7, 0xFFFFFFFF)])
def test_sort_stable_large(orc, n, mask):  # test.cpp:307-341, 366-400 (stability vs std::stable_sort)
    rng = np.random.default_rng(1)
    keys = (rng.integers(0, 1 << 32, size=n, dtype=np.uint64) & mask).astype(np.uint32)
    idx = np.arange(n, dtype=np.uint32)
    k, i = orc.sort_pairs(keys, idx)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(i, order.astype(np.uint32))
    assert np.array_equal(k, keys[order])


def test_apply_edit_known_answer(orc, golden):  # test.cpp:91-105
    v = golden["gpu_list_apply_edit"]["vectors"]
    assert orc.apply_edit(np.array(v["listData"]), np.array(v["editListData"])).tolist() == v["expectedResult"]


@pytest.mark.parametrize("name,list_a,list_b,n_hidden", [
    ("indexed_list_apply_hidden_edit_1", list(range(5)), [0, 1], 5),  # test.cpp:117-136
    ("indexed_list_apply_hidden_edit_2", list(range(5)), None, 5),    # test.cpp:138-160
    ("indexed_list_apply_hidden_edit_3", list(range(5)), None, 5),    # test.cpp:162-184
])
def test_hidden_edit_known_answers(orc, golden, name, list_a, list_b, n_hidden):
    v = golden[name]["vectors"]
    edit = np.array(v["editListData"])
    lb = list_b if list_b is not None else v["listBIdxData"]
    a, _ = orc.remap_index_list(np.array(list_a), edit, n_hidden)
    b, _ = orc.remap_index_list(np.array(lb), edit, n_hidden)
    assert a.tolist() == v["expectedResultA"]
    assert b.tolist() == v["expectedResultB"]


def test_delete_these_known_answers(orc, golden):
    # test.cpp:427-451: hidden [1..13]; list B covers hidden 0..10 and is deleted
    v = golden["delete_these_1"]["vectors"]
    hidden = np.array(v["hiddenValues"], np.uint32)
    edit = orc.delete_edit_list(13, np.arange(11))
    assert orc.apply_edit(hidden, edit).tolist() == v["expectedResult"]
    list_c, _ = orc.remap_index_list(np.array([0, 1, 2, 3, 4, 5, 6, 7, 11, 12]), edit, 13)
    assert list_c.tolist() == [0, 1]                                   # length C == 2
    assert orc.remap_index_list(np.arange(8), edit, 13)[0].size == 0  # length A == 0
    # test.cpp:453-464: everything deleted
    assert orc.delete_edit_list(13, np.arange(13)).size == 0
    # test.cpp:466-484: nothing deleted
    v3 = golden["delete_these_3"]["vectors"]
    e3 = orc.delete_edit_list(8, np.zeros(0, np.uint32))
    assert orc.apply_edit(np.array(v3["hiddenValues"]), e3).tolist() == v3["hiddenValues"]


def test_duplicate_these_known_answers(orc, golden):
    # test.cpp:486-511: duplicate hidden 0..2 of 10; lists B and C are remapped
    v = golden["duplicate_these"]["vectors"]
    edit = np.concatenate([np.arange(10), np.arange(3)])
    assert orc.apply_edit(np.array(v["hiddenValues"]), edit).tolist() == v["expectedHidden"]
    b, _ = orc.remap_index_list(np.arange(10), edit, 10)
    c, _ = orc.remap_index_list(np.arange(3, 10), edit, 10)
    assert b.tolist() == v["expectedListB"]
    assert c.tolist() == v["expectedListC"]
    # test.cpp:513-531: duplicating an empty list changes nothing
    ve = golden["duplicate_these_empty"]["vectors"]
    b2, _ = orc.remap_index_list(np.arange(5), np.arange(5), 5)
    assert b2.tolist() == ve["expectedResult"]
