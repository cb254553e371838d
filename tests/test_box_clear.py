"""The box-collision rejection test of the device (box_clear in apbf_internal.cuh)
never rules out a box that would push the particle: on random boxes, radii,
jitters in [0, 1] (both ends included) and positions within a few ulps of every
threshold, box_clear implies that the reference's push (box_collision.comp:35-57,
restated in FP32 with one rounding per operation) leaves the particle where it is."""
import numpy as np

f32 = np.float32


def smallest(v):
    b1, b2, b3 = v[0] <= v[1], v[0] <= v[2], v[1] <= v[2]
    return np.array([f32(1.0) if (b1 and b2) else f32(0.0), f32(1.0) if (not b1 and b3) else f32(0.0),
                     f32(1.0) if (not b2 and not b3) else f32(0.0)], f32)


def pushes(q, lo, hi, r, h1, h2):
    tmin = np.empty(3, f32)
    tmax = np.empty(3, f32)
    for c in range(3):
        bmin = f32(f32(lo[c] - r) - f32(h1[c] * f32(0.05)))
        bmax = f32(f32(hi[c] + r) + f32(h2[c] * f32(0.05)))
        tmin[c] = f32(bmin - q[c])
        tmax[c] = f32(bmax - q[c])
    m1 = smallest(-tmin)
    m2 = smallest(tmax)
    tmin = (tmin * m1).astype(f32)
    tmax = (tmax * m2).astype(f32)
    dmin = -f32(f32(tmin[0] + tmin[1]) + tmin[2])
    dmax = f32(f32(tmax[0] + tmax[1]) + tmax[2])
    return not (dmin <= 0.0 or dmax <= 0.0)


def box_clear(q, lo, hi, r):
    c = f32(0.0500001)
    b0 = [f32(f32(lo[d] - r) - c) for d in range(3)]
    b1 = [f32(f32(hi[d] + r) + c) for d in range(3)]
    if not max(abs(x) for x in b0 + b1) < 1e30:
        return False
    return any(q[d] < b0[d] for d in range(3)) or any(q[d] >= b1[d] for d in range(3))


def test_box_clear_is_conservative():
    rng = np.random.default_rng(7)
    with np.errstate(over="ignore", invalid="ignore"):
        checked = cleared = 0
        for _ in range(4000):
            scale = f32(10.0 ** rng.uniform(-1, 4))
            lo = (rng.uniform(-1, 1, 3) * scale).astype(f32)
            hi = (lo + rng.uniform(0.0, 2.0, 3) * scale).astype(f32)
            r = f32(rng.uniform(0.0, 3.0))
            h1 = rng.choice([0.0, 1.0, rng.uniform()], 3).astype(f32)
            h2 = rng.choice([0.0, 1.0, rng.uniform()], 3).astype(f32)
            # thresholds: the exact jittered ones and box_clear's, each +/- a few ulps
            cand = []
            for d in range(3):
                t = [f32(f32(lo[d] - r) - f32(h1[d] * f32(0.05))), f32(f32(hi[d] + r) + f32(h2[d] * f32(0.05))),
                     f32(f32(lo[d] - r) - f32(0.0500001)), f32(f32(hi[d] + r) + f32(0.0500001)),
                     f32(rng.uniform(lo[d] - 2 * scale, hi[d] + 2 * scale))]
                cand.append(t)
            for _k in range(12):
                q = np.empty(3, f32)
                for d in range(3):
                    base = cand[d][rng.integers(0, 5)]
                    q[d] = base
                    for _s in range(int(rng.integers(-3, 4)) % 7):
                        q[d] = np.nextafter(q[d], f32(np.inf) if rng.uniform() < 0.5 else f32(-np.inf), dtype=f32)
                checked += 1
                if box_clear(q, lo, hi, r):
                    cleared += 1
                    assert not pushes(q.copy(), lo, hi, r, h1, h2), (q, lo, hi, r, h1, h2)
        assert cleared > checked // 10  # the test exercises the rejection often
