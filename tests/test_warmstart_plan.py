"""The warm start's training mixture (bench.training_rollouts): rollouts of the dam
break, the adaptive water drop and the adaptive waterfall, about 60 M samples in
all, on seeds that neither a timed scene (seed = rank), a validation scene
(1000 + 10 rank + 3..6) nor the per-workload evaluation scene (3000) uses."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _samples(plan):
    import bench

    total = 0
    for w, seed, steps, every, n_end in plan:
        n0 = bench.make_spec(w).n
        records = (steps + every - 1) // every
        total += records * 0.5 * (n0 + n_end)  # a growing scene at its mean size
    return total


def test_mixture_covers_the_three_workloads_with_50m_samples():
    import bench

    plan = bench.training_rollouts(0)
    assert sorted({p[0] for p in plan}) == sorted(bench.MIXTURE)
    assert set(bench.MIXTURE) == {"dam_break_32k", "water_drop_250k", "waterfall_1m"}
    assert _samples(plan) >= 50e6
    # shares within a factor of two of each other
    per = {}
    for p in plan:
        per[p[0]] = per.get(p[0], 0) + _samples([p])
    assert max(per.values()) < 2 * min(per.values()), per


def test_mixture_seeds_are_held_out():
    import bench

    for world in (1, 2, 8):
        timed = set(range(world))
        valid = {1000 + 10 * r + k for r in range(world) for k in (3, 4, 5, 6)}
        train = {p[1] for r in range(world) for p in bench.training_rollouts(r)}
        assert not train & timed
        assert not train & valid
        assert 3000 not in train | valid | timed


def test_rollouts_reach_past_the_timed_window():
    import bench

    for w, seed, steps, every, _ in bench.training_rollouts(0):
        spec = bench.make_spec(w, seed=seed)
        assert steps >= spec.meta.get("presteps", 0) + 60 or steps == spec.substeps
