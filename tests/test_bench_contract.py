"""The benchmark's JSON contract on the CPU: the reference arm (the oracle,
every host core) runs without a GPU and prints one line with the keys the
driver reads."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    # the config-3 workload at 24^3 (the default 256^3 needs minutes per sample)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3", "--scale", "24"], capture_output=True,
                       text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert "workload" in line["config"]


def test_batch_cpu_schedule_longest_first():
    """The batched CPU baseline places solves longest first on the least
    loaded core: its wall time is the busiest core's total."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.lpt_makespan([5.0, 4.0, 3.0, 3.0, 3.0], 2) == 10.0
    assert bench.lpt_makespan([1.0] * 6, 3) == 2.0
    assert bench.lpt_makespan([7.0, 1.0], 16) == 7.0
    assert bench.lpt_makespan([], 4) == 0.0
