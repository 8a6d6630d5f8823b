"""CPU test of bench.py's reference arm (`--impl reference`): it runs the
reference's CPU implementation of the step on the host cores and prints one
JSON line with the same metric and workload as the GPU arm, marked as the
reference, with its CPU baseline and an end-to-end figure that moves no
bytes between host and device."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# Runs bench.py's main() in this interpreter, then reports which of the
# product's shared libraries the process mapped.
RUNNER = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("MAPPED", sorted(set(l.split()[-1] for l in maps.splitlines()
                           if l.endswith(".so") and "psyclonebench_gb300" in l)))
"""


def test_reference_arm_prints_its_json_line():
    out = subprocess.run([sys.executable, "-c", RUNNER],
                         cwd=REPO, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    # the reference arm maps no library of the product
    assert lines[-1] == "MAPPED []", lines[-1]
    line = json.loads(lines[-2])
    assert line["impl"] == "reference"
    assert line["metric"] == "Mcell-steps/s" and line["unit"] == "Mcell-steps/s"
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 3
    assert line["config"]["workload"] == "nemolite2d_fp64_4096x4096"
    # the same config object as the GPU arm's line
    sys.path.insert(0, REPO)
    import bench
    assert line["config"] == bench.bench_config(4096, 4104, 20.0)
    assert len(cb_layers := line["cpu_baseline"]["layers"]) == 2
    assert line["value"] == max(cb_layers.values())
    assert line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
