"""The CPU side of bench.py (no GPU): the reference arm runs the oracle on the
whole configured workload from a mesh built without the GPU library, and its
JSON line carries the contract's keys with the GPU line's `config`."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_runs_without_the_gpu_library():
    code = r"""
import json, sys
sys.argv = ["bench.py", "--impl", "reference", "--config", "c0", "--steps", "3", "--warmup", "1"]
sys.path.insert(0, ".")
import bench
bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"gpu_module": "lymph3d_apsc_gb300" in sys.modules,
                  "gpu_so_mapped": "liblymph3d_gb300" in maps,
                  "oracle_so_mapped": "liblymph_oracle_timing" in maps}))
"""
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    line, probe = lines[0], lines[1]
    assert not probe["gpu_module"] and not probe["gpu_so_mapped"] and probe["oracle_so_mapped"]
    assert line["impl"] == "reference" and line["unit"] == "DOF-steps/s" and line["value"] > 0
    assert line["steps"] == 3 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    cfg = line["config"]
    assert cfg["n_tet"] == 750 and cfg["n_poly"] == 125 and cfg["dofs"] == 125 * 30 and cfg["precision"] == "fp64"


def test_workload_config_is_the_same_for_both_arms():
    sys.path.insert(0, str(ROOT))
    import bench
    cfg = bench.CONFIGS["c2"]
    a = bench.workload_config(cfg, 384000, 46767, 35, 498457, "fp64", 1)
    b = bench.workload_config(cfg, 384000, 46767, 35, 498457, "fp64", 1)
    assert a == b and "p=4" in a["workload"] and "lognormal" in a["workload"]
