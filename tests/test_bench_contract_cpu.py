"""The benchmark's reference arm (the reference's CPU path on the host) runs
without a GPU and prints the one-line JSON contract the benchmark promises:
metric, value, unit and timing keys, the reference-arm marker, the CPU
baseline it measured and an end-to-end entry with zero device copies.  Run
here on a small signal (2^14 samples, J = 12)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
           "--warmup", "1", "--log2n", "14", "--levels", "12"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["higher_is_better"] is True and d["unit"] == "Gsamples/s"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("reference", "port")
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_roofline_byte_accounting():
    """Algorithmic bytes per forward+inverse step used for the HBM fractions:
    DWT 32 B per sample in FP64 (16 in FP32): each direction reads and writes
    the signal once; MODWT with J levels (1 + 2J) + (J + 2) values per sample
    (forward: the signal in, J scaling and J detail blocks out; inverse: s_J
    and J detail blocks in, the signal out), 312 B at J = 12 in FP64."""
    sys.path.insert(0, ROOT)
    import bench
    n = 1 << 20
    assert bench.step_bytes(0, n, 16, 8) == 32 * n
    assert bench.step_bytes(0, n, 16, 4) == 16 * n
    assert bench.step_bytes(1, n, 12, 8) == 312 * n
    assert bench.step_bytes(1, n, 12, 4) == 156 * n
    # smoothing adds, per golden step, two half-length inverses and the loss pass
    b = bench.smooth_bytes(1, n, 10, 2, 40, 8)
    h = n // 2
    assert b == bench.step_bytes(1, n, 10, 8) + 2 * (1 + 2 * 9) * h * 8 + \
        40 * (2 * (9 + 2) * h * 8 + n * 8 + 8 * n)
