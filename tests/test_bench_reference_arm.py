"""bench.py's reference arm (the reference's CPU step, timed on the host cores) runs from the
committed resolved-setup file and never maps the GPU library.  CPU only."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_does_not_load_the_gpu_library():
    code = (
        "import sys, json, runpy, io, contextlib\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']\n"
        "buf = io.StringIO()\n"
        "with contextlib.redirect_stdout(buf):\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'line': buf.getvalue().strip().splitlines()[-1], 'kzg': 'libkzg' in maps}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["kzg"] is False
    line = json.loads(out["line"])
    assert line["impl"] == "reference" and line["warmup"] == 0 and line["steps"] == 1
    assert "committed resolved-setup file" in line["cpu_baseline"]["sample"]
    assert line["value"] > 0
