"""The bench's reference arm (the reference step's CPU restatement on the host cores) keeps the
one-JSON-line contract on a machine without a GPU: same metric, unit, workload and configuration
as the GPU arm, impl "reference", its own cpu_baseline and an e2e object with no host-device
copies; and it builds its scene with the oracle's registration, loading nothing of the product."""
import json
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "body-steps/s"
    assert d["metric"] == "body-steps/s at 256k bodies" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["config"]["bodies"] == 262145 and "262,144 unit boxes" in d["config"]["workload"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]


def test_reference_arm_loads_no_product_library_and_shares_the_config():
    """The CPU arm maps oracle/liboracle.so only (no bullet3_gb300/libb3gpu.so), and its config
    equals the one the GPU arm builds for the same arguments."""
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--nx', '8'];"
        "import bench; a = bench.parse(); bench.reference_arm(a);"
        "maps = open('/proc/self/maps').read();"
        "print(json.dumps({'gpu_lib': 'libb3gpu.so' in maps, 'oracle_lib': 'liboracle.so' in maps,"
        " 'config': bench.bench_config(a, bench.make_scene(a))}))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.strip()]
    arm, probe = lines[0], lines[1]
    assert probe["gpu_lib"] is False and probe["oracle_lib"] is True
    assert arm["config"] == probe["config"]
