"""bench.py --impl reference on the CPU: the reference arm renders the
workload's own configuration with the CPU port of the path (no GPU, no CUDA
library), prints one JSON line whose config is the GPU arm's, and maps no
libsolrt.so into its process."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--workload", "cornell", "--steps", "2", "--warmup", "1"]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit:
    pass
maps = open("/proc/self/maps").read()
print("MAPPED", "libsolrt" in maps, "liboracle" in maps)
"""


def test_reference_arm_line():
    r = subprocess.run([sys.executable, "-c", PROBE], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Mrays/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the GPU arm's config object for the same workload, key for key
    cfg = d["config"]
    assert cfg["workload"].startswith("procedural Cornell box 32 tris, 256x256, 16 spp")
    assert cfg["width"] == 256 and cfg["spp"] == 16 and cfg["max_depth"] == 5
    assert cfg["parallelism"] == "single" and cfg["bvh"] == "bvh2+sah" and "l2" in cfg
    mapped = [l for l in r.stdout.splitlines() if l.startswith("MAPPED")][0].split()
    assert mapped[1] == "False", "the reference arm loaded the CUDA library"
    assert mapped[2] == "True"
