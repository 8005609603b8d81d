"""bench.py --impl reference runs the reference's own host path (numpy
normals, Camera matrices, host LUTs, the oracle): it prints the contract's
line and loads neither torch nor the pyvr_gb300 CUDA library."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import sys, io, contextlib, json
sys.argv = ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "1", "--cpu-seconds", "1",
            "--serving-volumes", "4", "--serving-extra", "4", "--serving-min-dim", "24",
            "--serving-max-dim", "40"]
sys.path.insert(0, ROOT)
import bench
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    bench.main()
libs = sorted({l.split()[-1] for l in open("/proc/self/maps") if ".so" in l})
print(json.dumps({"line": buf.getvalue().strip(), "libs": libs, "torch": "torch" in sys.modules}))
"""


def test_reference_arm_is_the_reference_host_path():
    out = subprocess.run([sys.executable, "-c", PROBE.replace("ROOT", repr(ROOT))], cwd=ROOT,
                         capture_output=True, text=True, timeout=600, check=True).stdout
    res = json.loads(out.strip().splitlines()[-1])
    line = json.loads(res["line"])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "renders/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert not res["torch"]
    assert not any("libpyvr_gb300" in l for l in res["libs"]), res["libs"]
    assert any("libpvr_oracle" in l for l in res["libs"])
