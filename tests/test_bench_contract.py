"""bench.py's JSON contract, on the CPU: the reference arm (the CPU baseline
of the path, no GPU needed) prints one JSON line with the benchmark keys."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def test_reference_arm_serving_line():
    """The default workload's reference arm: small graphs, CPU only, and the
    engine's library never mapped into the process."""
    d = _run("--impl", "reference", "--serving-scales", "10,11,12,13", "--requests", "60", "--steps", "2",
             "--warmup", "1", "--cpu-seconds", "1")
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == "served queries/s" and d["unit"] == "queries/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["config"]["workload"] == "serving-rmat10-11-12-13-24GiB"
    assert sum(d["config"]["mix"].values()) == 60
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1


def test_reference_arm_loads_no_engine_library():
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--serving-scales', '10,11,12,13', "
            "'--requests', '40', '--steps', '1', '--warmup', '1', '--cpu-seconds', '1']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('ENGINE_MAPPED' if 'libog.so' in maps else 'ENGINE_NOT_MAPPED')")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "ENGINE_NOT_MAPPED" in out.stdout


def test_reference_arm_sssp_line():
    d = _run("--impl", "reference", "--workload", "sssp-oom", "--scale", "12", "--steps", "2", "--warmup", "1",
             "--cpu-seconds", "1")
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["metric"] == "queries/s" and d["unit"] == "queries/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["e2e"] == {"value": d["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert d["config"]["workload"].startswith("oom-sssp-rmat12")
    assert d["config"]["sssp_delta"] == 4.0  # the engine's default, as in the GPU arm


def test_help_lists_workloads():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], cwd=ROOT,
                         capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    for w in ("sssp-oom", "cc-oom", "bfs-batch", "bfs-resident", "pr-precision", "serving"):
        assert w in out.stdout


def test_config_legs_parse():
    """Every configuration the default line runs after the serving passes is
    a valid bench.py command line (a renamed workload would drop a leg)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    keys = set()
    for key, argv in bench.CONFIG_LEGS:
        old = sys.argv
        try:
            sys.argv = ["bench.py", *argv, "--warmup", "3", "--configs", "none"]
            a = bench.parse_args()
        finally:
            sys.argv = old
        assert a.workload == key and a.warmup == 3 and a.configs == "none"
        keys.add(key)
    assert keys == {"bfs-resident", "sssp-oom", "cc-oom", "pr-precision", "bfs-batch"}
