"""bench.py --impl reference runs the CPU restatement of the reference's shader math
on every host core and never maps the library under test (libapbf_gb300.so), in
the parent process or in any replica."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_maps_no_product_library():
    env = dict(os.environ)
    env.pop("RANK", None)
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload",
                          "dam_break_32k", "--steps", "1", "--warmup", "3"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(next(l for l in out.stdout.splitlines() if l.startswith("{")))
    assert line["impl"] == "reference"
    assert line["config"]["product_library_mapped"] is False
    assert all("libapbf_oracle" in lib for lib in line["config"]["oracle_library"])
    assert line["value"] > 0 and line["cpu_baseline"]["cores"] == os.cpu_count()
    # a bounded sample: 1/8 of the scene's particles per replica
    assert line["config"]["sample_scale"] == 0.125 and line["config"]["sample_particles"] == 16 ** 3


def test_samples_scale_with_their_workload():
    """A bounded sample of a workload has about the requested fraction of its particles
    (the reference arm and the CPU baseline time such samples)."""
    sys.path.insert(0, str(ROOT))
    import bench

    for w in ("dam_break_32k", "water_drop_250k", "water_drop_250k_plain", "waterfall_1m"):
        full = bench.make_spec(w).n
        for scale in (1.0 / 8.0, 1.0 / 64.0):
            n = bench.make_spec(w, scale=scale).n
            assert 0.5 * scale * full <= n <= 2.0 * scale * full, (w, scale, n, full)
