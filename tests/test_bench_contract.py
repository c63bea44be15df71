"""The bench's workload and its reference arm, on the CPU.

* the headline workload: 4096 even sizes in [16, 256], seeded and reproducible,
  sum of 8 n^2 about 766 MB (the size the headline configuration is quoted on);
* packed inputs: column-major, back to back, every matrix exactly skew-symmetric,
  entries of (B - B^T)/2 with B ~ N(0, 1/n);
* the algorithmic flops of one step (4/3 n^3 + 2 n^3 per matrix);
* `bench.py --impl reference` prints one JSON line with the keys the reference arm
  must carry (impl, metric, value, unit, cpu_baseline, e2e with no host transfers),
  on the headline metric and configuration, and exits 0.
"""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_workload_sizes():
    s = bench.workload_sizes()
    assert len(s) == bench.COUNT == 4096
    assert np.all(s % 2 == 0) and s.min() >= 16 and s.max() <= 256
    np.testing.assert_array_equal(s, bench.workload_sizes())
    assert not np.array_equal(s, bench.workload_sizes(rank=1))  # replicas get their own matrices
    total_bytes = float((8 * s.astype(np.float64) ** 2).sum())
    assert 0.74e9 < total_bytes < 0.79e9


def test_packed_inputs_are_skew():
    sizes = np.array([16, 2, 40, 256, 18], dtype=np.int64)
    buf, offs = bench.packed_inputs(sizes)
    assert buf.size == int((sizes ** 2).sum())
    np.testing.assert_array_equal(offs, np.concatenate([[0], np.cumsum(sizes[:-1] ** 2)]))
    for b, n in enumerate(sizes):
        A = buf[offs[b]:offs[b] + n * n].reshape(n, n, order="F")
        np.testing.assert_array_equal(A, -A.T)
        # (B - B^T)/2 with B ~ N(0, 1/n): off-diagonal variance 1/(2n)
        if n >= 40:
            off = A[np.triu_indices(n, 1)]
            assert 0.5 / (2 * n) < off.var() < 2.0 / (2 * n)


def test_step_flops():
    s = bench.workload_sizes()
    flops = float(bench.flops_per_matrix(s).sum())
    n = s.astype(np.float64)
    assert abs(flops - float((10.0 / 3.0 * n ** 3).sum())) <= 1e-9 * flops
    assert 6.0e10 < flops < 6.2e10


def test_reference_arm_line():
    env = dict(os.environ)
    env.setdefault("OMP_NUM_THREADS", "2")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--cpu-sample", "24"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT and d["higher_is_better"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["config"]["workload"].startswith("batched_logabspf_grad_4096x")
