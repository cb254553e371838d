"""bench.py's N>1 path (independent replicas, one per rank) on CPU with two gloo ranks:
the whole-job figures are the slowest rank's time and the particle-substeps of all
ranks, the same on every rank; each rank's scene is seeded by its rank; the
reference arm runs on rank 0 only."""
import os
import socket
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t, p = bench.reduce_over_ranks(10.0 + 5.0 * rank, 100.0 * (rank + 1), dist, "cpu")
    # the batch's comparison runs: each rank its own scene table and timings
    w = bench.batch_whole_job(seq_ms=20.0 * (rank + 1), seq_particles=1000.0 * (rank + 1), e2e_s=0.5 + rank,
                              e2e_particles=300.0, scenes=64, particles=5000 + rank, dist=dist, device="cpu")
    out.put((rank, t, p, w))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_aggregate_slowest_time_and_all_particles():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=120) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
    assert [p.exitcode for p in procs] == [0, 0]
    assert [r[:3] for r in res] == [(0, 15.0, 300.0), (1, 15.0, 300.0)]
    # batch: every whole-job field is the same on both ranks: slowest time, all ranks' work
    for _, _, _, w in res:
        assert w["sequential_ms"] == 40.0
        assert w["sequential_value"] == 3000.0 / 0.040
        assert w["e2e_value"] == 600.0 / 1.5
        assert w["scenes"] == 128 and w["particles_total"] == 10001


def test_one_process_is_unchanged():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reduce_over_ranks(12.5, 40.0, None, "cpu") == (12.5, 40.0)


def test_scenes_are_seeded_by_rank():
    sys.path.insert(0, str(ROOT))
    import bench

    a = bench.make_spec("dam_break_32k", seed=0).state["position"]
    b = bench.make_spec("dam_break_32k", seed=1).state["position"]
    assert a.shape == b.shape and not np.array_equal(a, b)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("RANK", "1")
    args = SimpleNamespace(workload="dam_break_32k", steps=1, warmup=3, gpus=2, oracle_variant="f32")
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
