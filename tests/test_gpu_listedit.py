"""The list-edit services against the reference's own known answers (source/
test.cpp) and the oracle on random lists."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(a):
    import torch

    return torch.from_numpy(np.asarray(a, np.uint32).view(np.int32)).cuda()


def _np(t):
    return t.cpu().numpy().view(np.uint32)


@pytest.fixture(scope="module")
def ctx():
    from apbf_gb300.api import Context

    c = Context(particle_capacity=300_000, max_neighbors=8, max_log2res=3)
    yield c
    c.close()


def test_apply_edit_known_answer(golden):  # test.cpp:91-105
    from apbf_gb300.api import lists

    v = golden["gpu_list_apply_edit"]["vectors"]
    assert _np(lists.apply_edit(_t(v["listData"]), _t(v["editListData"]))).tolist() == v["expectedResult"]


@pytest.mark.parametrize("name,list_a,list_b,n_hidden", [
    ("indexed_list_apply_hidden_edit_1", list(range(5)), [0, 1], 5),  # test.cpp:117-136
    ("indexed_list_apply_hidden_edit_2", list(range(5)), None, 5),    # test.cpp:138-160
    ("indexed_list_apply_hidden_edit_3", list(range(5)), None, 5),    # test.cpp:162-184
])
def test_remap_known_answers(ctx, golden, name, list_a, list_b, n_hidden):
    from apbf_gb300.api import lists

    v = golden[name]["vectors"]
    edit = _t(v["editListData"])
    lb = list_b if list_b is not None else v["listBIdxData"]
    a, _, _ = lists.remap_index(ctx, _t(list_a), edit, n_hidden)
    b, _, _ = lists.remap_index(ctx, _t(lb), edit, n_hidden)
    assert _np(a).tolist() == v["expectedResultA"]
    assert _np(b).tolist() == v["expectedResultB"]


def test_delete_and_duplicate_known_answers(ctx, golden):
    from apbf_gb300.api import lists

    # test.cpp:427-451
    v = golden["delete_these_1"]["vectors"]
    edit = lists.delete_edit(ctx, _t(np.arange(11)), 13)
    assert _np(lists.apply_edit(_t(v["hiddenValues"]), edit)).tolist() == v["expectedResult"]
    c, _, _ = lists.remap_index(ctx, _t([0, 1, 2, 3, 4, 5, 6, 7, 11, 12]), edit, 13)
    assert _np(c).tolist() == [0, 1]
    assert lists.remap_index(ctx, _t(np.arange(8)), edit, 13)[0].numel() == 0
    # test.cpp:453-464 and 466-484
    assert lists.delete_edit(ctx, _t(np.arange(13)), 13).numel() == 0
    v3 = golden["delete_these_3"]["vectors"]
    e3 = lists.delete_edit(ctx, _t(np.zeros(0)), 8)
    assert _np(lists.apply_edit(_t(v3["hiddenValues"]), e3)).tolist() == v3["hiddenValues"]
    # test.cpp:486-511: duplicating hidden 0..2 of 10
    vd = golden["duplicate_these"]["vectors"]
    dup = _t(np.concatenate([np.arange(10), np.arange(3)]))
    assert _np(lists.apply_edit(_t(vd["hiddenValues"]), dup)).tolist() == vd["expectedHidden"]
    assert _np(lists.remap_index(ctx, _t(np.arange(10)), dup, 10)[0]).tolist() == vd["expectedListB"]
    assert _np(lists.remap_index(ctx, _t(np.arange(3, 10)), dup, 10)[0]).tolist() == vd["expectedListC"]
    ve = golden["duplicate_these_empty"]["vectors"]
    assert _np(lists.remap_index(ctx, _t(np.arange(5)), _t(np.arange(5)), 5)[0]).tolist() == ve["expectedResult"]


def test_append_known_answers(golden):  # test.cpp:47-89
    import torch

    from apbf_gb300.api import lists

    v = golden["gpu_list_concatenation_1"]["vectors"]
    dst = torch.zeros(16, dtype=torch.int32, device="cuda")
    dst[:4] = _t(v["listAData"])
    n = torch.tensor([4], dtype=torch.int32, device="cuda")
    lists.append(dst, n, _t(v["listBData"]), torch.tensor([3], dtype=torch.int32, device="cuda"))
    assert int(n.item()) == 7
    assert _np(dst[:7]).tolist() == v["listAData"] + v["listBData"]
    e = golden["gpu_list_append_empty"]["vectors"]
    dst2 = torch.zeros(8, dtype=torch.int32, device="cuda")
    dst2[:4] = _t(e["listAData"])
    n2 = torch.tensor([4], dtype=torch.int32, device="cuda")
    lists.append(dst2, n2, _t([0]), torch.tensor([0], dtype=torch.int32, device="cuda"))
    assert int(n2.item()) == 4 and _np(dst2[:4]).tolist() == e["listAData"]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_lists_match_oracle(ctx, orc, seed):
    from apbf_gb300.api import lists

    rng = np.random.default_rng(seed)
    n_hidden = int(rng.integers(1000, 200_000))
    index_list = rng.integers(0, n_hidden, size=int(rng.integers(0, 150_000))).astype(np.uint32)
    deleted = np.unique(rng.integers(0, n_hidden, size=n_hidden // 3)).astype(np.uint32)
    edit = lists.delete_edit(ctx, _t(deleted), n_hidden)
    e_or = orc.delete_edit_list(n_hidden, deleted)
    assert np.array_equal(_np(edit), e_or)
    out, pos, req = lists.remap_index(ctx, _t(index_list), edit, n_hidden)
    o_or, p_or = orc.remap_index_list(index_list, e_or, n_hidden)
    assert req == o_or.size and np.array_equal(_np(out), o_or) and np.array_equal(_np(pos), p_or)
    # a duplication with repeated ids
    dup = np.concatenate([np.arange(n_hidden), rng.integers(0, n_hidden, size=5000)]).astype(np.uint32)
    out2, pos2, _ = lists.remap_index(ctx, _t(index_list), _t(dup), n_hidden)
    o2, p2 = orc.remap_index_list(index_list, dup, n_hidden)
    assert np.array_equal(_np(out2), o2) and np.array_equal(_np(pos2), p2)
    vals = rng.integers(0, 2**32, size=(n_hidden, 3), dtype=np.uint64).astype(np.uint32)
    got = _np(lists.apply_edit(_t(vals.ravel()), _t(dup), stride_words=3)).reshape(-1, 3)
    assert np.array_equal(got, orc.apply_edit(vals, dup, stride_words=3).reshape(-1, 3))
