"""The validation rule that picks the warm-start network and its over-relaxation
bound (warmstart.select_warm_start), on fake contexts whose outcomes are set per
solve form: admissibility (every counted substep converged, final mean |v|^2 and
99th-percentile height within the slacks of the largest converging plain rule),
fewest particle-weighted passes, ties to the smaller bound, the fallback to no
warm start, and the slacks switched off."""
import numpy as np
import pytest
import torch

from apbf_gb300 import _native as N
from apbf_gb300.warmstart import ValidationCase, run_case, select_warm_start

FIX = 262144.0
LEARNED = N.WARM_LEARNED | N.WARM_PROJECTED


class FakeStatus:
    def __init__(self, passes, converged):
        self.density_passes = passes
        self.converged_substeps = converged


class FakeCtx:
    """Counts substeps; reports `passes` per substep and `converged` of the counted
    ones; ends with every particle at speed sqrt(v2) and height y."""

    def __init__(self, outcome, n):
        self.passes, self.conv_frac, self.v2, self.y = outcome
        self.n = n
        self.steps = 0
        self.closed = False

    def substep(self, dt):
        self.steps += 1

    def check_status(self):
        s, self.steps = self.steps, 0
        return FakeStatus(int(round(self.passes * s)), int(round(self.conv_frac * s)))

    def lengths(self):
        return self.n, 0

    def fluid_view(self):
        v = torch.zeros((self.n, 4), dtype=torch.float32)
        v[:, 0] = float(np.sqrt(self.v2))
        p = torch.zeros((self.n, 4), dtype=torch.int32)
        p[:, 1] = int(self.y * FIX)
        return {"velocity": v, "position": p}

    def close(self):
        self.closed = True


class FakeNet:
    """Parameter vector [id, omega, min_neighbors]: what a context is loaded with."""

    def __init__(self, ident):
        self.params = torch.tensor([float(ident), 0.0, 0.0])

    @property
    def omega_max(self):
        return float(self.params[1])

    @omega_max.setter
    def omega_max(self, v):
        self.params[1] = float(v)

    @property
    def min_neighbors(self):
        return float(self.params[2])

    @min_neighbors.setter
    def min_neighbors(self, v):
        self.params[2] = float(v)


def _case(table, n=1000, before=3, counted=10):
    """table: {"reference": outcome, "projected": outcome, (net id, omega): outcome};
    outcome = (passes per substep, converged fraction, mean v^2, height)."""
    made = []

    def make(mode, params):
        if mode == 0:
            out = table["reference"]
        elif mode == N.WARM_PROJECTED:
            out = table["projected"]
        else:
            assert mode == LEARNED
            out = table[(int(params[0]), float(params[1]))]
        ctx = FakeCtx(out, n)
        made.append(ctx)
        return ctx

    return ValidationCase(make=make, dt=1.0 / 240.0, before=before, counted=counted), made


PLAIN = {"reference": (24.0, 1.0, 100.0, 70.0), "projected": (37.0, 1.0, 40.0, 60.0)}


def test_run_case_measures_the_counted_window():
    case, made = _case({**PLAIN}, n=500, before=4, counted=8)
    r = run_case(case, 0)
    assert r == {"passes": 24.0, "converged": 8, "mean_v2": pytest.approx(100.0), "y_p99": pytest.approx(70.0),
                 "particles": 500}
    assert made[0].closed


def test_fewest_passes_among_admissible_ties_to_smaller_bound():
    # bounds: energy 1.05 x 100 = 105, height 1.25 x 70 = 87.5 (the reference rule is the larger)
    t = {**PLAIN,
         (0, 2.0): (18.0, 1.0, 90.0, 80.0),    # admissible
         (0, 3.0): (14.0, 1.0, 104.0, 84.0),   # admissible
         (0, 4.0): (12.0, 1.0, 110.0, 85.0),   # too energetic
         (1, 2.0): (14.0, 1.0, 95.0, 80.0),    # admissible, ties (0, 3.0) with a smaller bound
         (1, 3.0): (13.0, 1.0, 100.0, 90.0),   # splashes too high
         (1, 4.0): (11.0, 0.9, 50.0, 60.0)}    # misses the target in one substep
    case, _ = _case(t)
    nets = {"a": FakeNet(0), "b": FakeNet(1)}
    choice, table = select_warm_start(nets, [case], (2.0, 3.0, 4.0), min_neighbors=12.0)
    assert choice["net"] == "b" and choice["omega_max"] == 2.0 and choice["min_neighbors"] == 12.0
    assert float(choice["params"][0]) == 1.0 and float(choice["params"][1]) == 2.0
    assert (nets["b"].omega_max, nets["b"].min_neighbors) == (2.0, 12.0)
    adm = {k: v["admissible"] for k, v in table["candidates"].items()}
    assert adm == {"a / omega 2": True, "a / omega 3": True, "a / omega 4": False,
                   "b / omega 2": True, "b / omega 3": False, "b / omega 4": False}
    assert table["energy_bound"] == [pytest.approx(105.0)] and table["height_bound"] == [pytest.approx(87.5)]
    assert table["candidates"]["a / omega 4"]["energy_ratio"] == [1.1]


def test_bound_comes_from_the_converging_plain_rule():
    # the reference rule misses the target: the projected rule (v2 40, y 60) sets the bounds
    t = {"reference": (100.0, 0.0, 1000.0, 300.0), "projected": (21.0, 1.0, 40.0, 60.0),
         (0, 2.0): (16.0, 1.0, 45.0, 70.0),    # 1.125 x energy: out
         (0, 3.0): (19.0, 1.0, 41.0, 74.0)}    # within 1.05 x 40 and 1.25 x 60
    case, _ = _case(t)
    choice, table = select_warm_start({"a": FakeNet(0)}, [case], (2.0, 3.0))
    assert choice["omega_max"] == 3.0
    assert table["energy_bound"] == [pytest.approx(42.0)]


def test_no_admissible_candidate_and_slacks_off():
    t = {**PLAIN, (0, 2.0): (12.0, 1.0, 300.0, 200.0), (0, 3.0): (10.0, 1.0, 500.0, 400.0)}
    case, _ = _case(t)
    net = FakeNet(0)
    net.omega_max, net.min_neighbors = 7.0, 9.0
    choice, table = select_warm_start({"a": net}, [case], (2.0, 3.0))
    assert choice is None and not any(v["admissible"] for v in table["candidates"].values())
    assert (net.omega_max, net.min_neighbors) == (7.0, 9.0)  # left as it came
    choice, _ = select_warm_start({"a": FakeNet(0)}, [case], (2.0, 3.0), energy_slack=0.0, height_slack=0.0)
    assert choice["omega_max"] == 3.0  # only convergence is left to check


def test_passes_are_weighted_by_particles():
    big = {**PLAIN, (0, 2.0): (10.0, 1.0, 90.0, 70.0), (0, 3.0): (12.0, 1.0, 90.0, 70.0)}
    small = {**PLAIN, (0, 2.0): (30.0, 1.0, 90.0, 70.0), (0, 3.0): (12.0, 1.0, 90.0, 70.0)}
    c1, _ = _case(big, n=9000)
    c2, _ = _case(small, n=1000)
    choice, table = select_warm_start({"a": FakeNet(0)}, [c1, c2], (2.0, 3.0))
    # omega 2: (9000 * 10 + 1000 * 30) / 10000 = 12.0; omega 3: 12.0 -> tie, the smaller bound
    assert table["candidates"]["a / omega 2"]["passes"] == pytest.approx(12.0)
    assert choice["omega_max"] == 2.0
    c2b, _ = _case({**small, (0, 2.0): (31.0, 1.0, 90.0, 70.0)}, n=1000)
    choice, _ = select_warm_start({"a": FakeNet(0)}, [c1, c2b], (2.0, 3.0))
    assert choice["omega_max"] == 3.0
