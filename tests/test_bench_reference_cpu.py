"""The CPU reference arm of bench.py: one JSON line in the metric's unit, and
the process never loads the product library (its inputs come from the
oracle's own generator)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import io, json, sys, contextlib
sys.argv = ["bench.py", "--impl", "reference", "--workload", "rmat-u-100k", "--n", "100000",
            "--m", "1000000", "--sources", "200", "--parts", "4", "--steps", "2", "--warmup", "1"]
sys.path.insert(0, %r)
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.main()
maps = open("/proc/self/maps").read()
print(json.dumps({"out": buf.getvalue(), "loaded_product": "libtsvd_gb300" in maps,
                  "modules": sorted(m for m in sys.modules if "tsvd" in m)}))
"""


def test_reference_arm_line_without_the_product_library():
    r = subprocess.run([sys.executable, "-c", PROBE % ROOT], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert not res["loaded_product"], res
    assert "tsvd_gb300" not in res["modules"], res["modules"]
    line = json.loads(res["out"].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "edge updates/s"
    assert line["value"] > 0 and line["steps"] >= 1
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert line["e2e"]["h2d_bytes_per_step"] == 0
