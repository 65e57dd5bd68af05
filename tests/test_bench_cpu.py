"""bench.py pieces that run without a GPU: the reference arm's JSON line and
the roofline work model."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "3000",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "cpu_baseline", "e2e", "dtype", "config"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "particle-steps/s"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("port", "reference")


class _FakeSim:
    n, k = 400, 32

    def state(self):
        r = np.random.default_rng(1)
        return {k: r.random(self.n) for k in ["x", "y", "vx", "vy", "u", "ax", "ay", "udot"]}

    def neighbours(self):
        r = np.random.default_rng(2)
        ids = r.integers(0, self.n, (self.n, self.k))
        d = np.sort(r.random((self.n, self.k)), axis=1)[:, ::-1]
        img = r.integers(0, 9, (self.n, self.k)).astype(np.int32)
        return ids, d, img


def test_pair_statistics_and_work_model():
    lo, visc = bench.pair_statistics(_FakeSim(), 1e-5)
    assert 0.3 < lo < 0.7 and 0.3 < visc < 0.7
    w = bench.algorithmic(32, 8.9, 8.9, lo, visc)
    assert w["force_integrate"]["fp64_slots"] > w["density"]["fp64_slots"] > 0
    # every approaching pair adds the viscosity work, two divisions included
    w0 = bench.algorithmic(32, 8.9, 8.9, lo, 0.0)
    w1 = bench.algorithmic(32, 8.9, 8.9, lo, 1.0)
    assert abs((w1["force_integrate"]["fp64_slots"] - w0["force_integrate"]["fp64_slots"]) - 32 * (16 + 2 * 8.9)) < 1e-9
