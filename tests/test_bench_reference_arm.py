"""bench.py's reference arm (the CPU port of the reference kernels, no GPU) prints one JSON
line with the keys the benchmark contract asks for."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--cells", "256",
                          "--steps", "1", "--warmup", "0", "--cpu-iters", "2"], check=True, capture_output=True,
                         text=True, cwd=ROOT, timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("CG cell-iterations/s")
    assert d["unit"] == "cell-iterations/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"]


def test_reference_arm_config_equals_gpu_arm():
    """Both arms print the same config dict for the same arguments; the CPU sample window is
    reported outside it."""
    sys.path.insert(0, ROOT)
    import bench

    for solver in ("cg", "ppcg"):
        argv = ["--impl", "reference", "--solver", solver, "--cells", "128", "--steps", "1", "--warmup", "0",
                "--iters", "7", "--cpu-iters", "3"]
        out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + argv, check=True,
                             capture_output=True, text=True, cwd=ROOT, timeout=600).stdout
        d = json.loads([ln for ln in out.splitlines() if ln.startswith("{")][0])
        gpu_args = bench.parse(argv[2:])
        assert d["config"] == bench.config_json(gpu_args, 1)
        assert d["metric"] == bench.metric_name(gpu_args)
        assert d["cpu_sample"]["iterations_per_step"] == 3
