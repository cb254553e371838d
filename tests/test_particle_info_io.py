"""save_particle_info files read back on the host: load_particle_info parses the
';'-separated lists and data.csv as the exporter writes them (std::ostream's six
significant digits), and state_from_particle_info rebuilds an uploadable state from
data.csv whose fields agree with the written one to that precision."""
import numpy as np
import pytest

from apbf_gb300 import scenes
from apbf_gb300.api import PARTICLE_INFO_COLUMNS, load_particle_info, state_from_particle_info


def _g(x) -> str:
    return format(float(np.float32(x)), "g")  # std::ostream default: %g, 6 significant digits


def _write(folder, st, center=(0.0, 10.0, -60.0)):
    """The exporter's files for a state (the same formulas and formatting)."""
    p = st["position"][:, :3].astype(np.float32) / np.float32(262144.0)
    cd = np.sqrt(np.sum((p - np.float32(center)) ** 2, axis=1, dtype=np.float32))
    bd = st["boundary_distance"].astype(np.float32) / np.float32(262144.0)
    cnt = np.arange(p.shape[0]) % 7
    lists = {"centerDist": cd, "radius": st["radius"], "neighborCount": cnt, "kernelWidth": st["kernel_width"],
             "targetRadius": st["target_radius"], "boundaryDistance": bd}
    for name, v in lists.items():
        (folder / f"{name}.txt").write_text("".join((str(int(x)) if name == "neighborCount" else _g(x)) + ";"
                                                    for x in v))
    order = np.argsort(cd, kind="stable")
    rows = [",".join([_g(cd[i]), _g(bd[i]), _g(st["kernel_width"][i]), str(int(cnt[i])), _g(st["radius"][i]),
                      _g(st["target_radius"][i]), _g(st["inverse_mass"][i]), _g(p[i, 0]), _g(p[i, 1]), _g(p[i, 2])])
            for i in order]
    (folder / "data.csv").write_text(",".join(PARTICLE_INFO_COLUMNS) + "\n" + "\n".join(rows) + "\n")
    return lists, order


def test_load_lists_and_table(tmp_path):
    rng = np.random.default_rng(4)
    st = scenes.make_state(scenes.lattice([5, 5, 5], [6, 5, 4], 2.0, 0.3, rng))
    st["boundary_distance"] = rng.integers(0, 40 * 262144, size=st["radius"].shape[0]).astype(np.uint32)
    lists, order = _write(tmp_path, st)
    got = load_particle_info(tmp_path)
    for name, v in lists.items():
        assert got[name].shape == v.shape, name
        if name == "neighborCount":
            assert np.array_equal(got[name], v)
        else:
            assert np.allclose(got[name], v, rtol=1e-5, atol=1e-6), name
    d = got["data"]
    assert set(d) == set(PARTICLE_INFO_COLUMNS)
    assert np.all(np.diff(d["center distance"]) >= 0)
    assert np.array_equal(d["neighbor count"], lists["neighborCount"][order])


def test_state_from_data_csv(tmp_path):
    rng = np.random.default_rng(5)
    st = scenes.make_state(scenes.lattice([5, 5, 5], [5, 5, 5], 2.0, 0.3, rng), radius=1.5)
    st["boundary_distance"] = rng.integers(0, 40 * 262144, size=st["radius"].shape[0]).astype(np.uint32)
    _, order = _write(tmp_path, st)
    back = state_from_particle_info(tmp_path)
    assert set(back) == set(st)
    for k in ("radius", "target_radius", "kernel_width", "inverse_mass"):
        assert np.allclose(back[k], st[k][order], rtol=1e-5), k
    x0 = st["position"][order, :3].astype(np.float64)
    assert np.all(np.abs(back["position"][:, :3] - x0) <= 1e-5 * np.abs(x0) + 2), "positions to 6 digits"
    assert np.all(np.abs(back["boundary_distance"].astype(np.int64) - st["boundary_distance"][order]) <=
                  1e-5 * st["boundary_distance"][order] + 2)
    assert np.array_equal(back["pos_backup"], back["position"]) and not back["velocity"].any()


def test_unexpected_columns_rejected(tmp_path):
    (tmp_path / "data.csv").write_text("a,b\n1,2\n")
    with pytest.raises(ValueError):
        load_particle_info(tmp_path)
