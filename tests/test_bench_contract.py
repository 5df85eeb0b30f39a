"""The reference arm of bench.py (the CPU restatement of the reference's run_many
on the host's cores) prints the JSON line the benchmark contract asks for; it
needs no GPU, so the contract is checked here on a small DAG."""
from __future__ import annotations

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    env = dict(os.environ, MCD_REF_STEP_SECONDS="0.3")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--layers", "20"], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == line["metric"] == "sample-edges/s"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["steps"] == 2
    cfg = line["config"]
    assert cfg["events"] == 2000 and cfg["samples_per_step"] == 19456 and cfg["levels"] > 1
    assert set(cfg) == {"workload", "events", "links", "preds", "levels", "samples_per_step", "outputs"}
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_maps_no_product_library():
    """The reference arm times the oracle only: the GPU engine's libraries (and
    torch) stay out of its process."""
    probe = (
        "import sys, runpy\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--layers', '10']\n"
        "try:\n"
        "    runpy.run_path('bench.py', run_name='__main__')\n"
        "except SystemExit:\n"
        "    pass\n"
        "maps = open('/proc/self/maps').read()\n"
        "bad = [m for m in ('libmcdagprop_gb300', 'mc_dagprop_gb300/_core') if m in maps]\n"
        "print('MAPPED', bad, 'torch' in sys.modules, 'mc_dagprop_gb300' in sys.modules)\n"
    )
    env = dict(os.environ, MCD_REF_STEP_SECONDS="0.2")
    out = subprocess.run([sys.executable, "-c", probe], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    last = [ln for ln in out.stdout.splitlines() if ln.startswith("MAPPED")][-1]
    assert last == "MAPPED [] False False", last
