"""The benchmark's reference arm on the CPU: `bench.py --impl reference` runs the
reference's own CPU path (the shim-built reference where it was compiled, else the
oracle port) on a bounded sample and prints one JSON line with the contract's keys,
without touching a GPU or the product library."""

from __future__ import annotations

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# runs bench.py's main in this process, then reports whether the product's shared objects were mapped
_DRIVER = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-seconds", "1"]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("PRODUCT-LOADED" if ("libragnar_gb300" in maps or "ragnar_gb300/_ragnar" in maps) else "PRODUCT-NOT-LOADED")
"""


def test_reference_arm_prints_the_contract_line():
    proc = subprocess.run([sys.executable, "-c", _DRIVER], cwd=ROOT, capture_output=True, text=True, timeout=300,
                          check=True)
    out = proc.stdout.strip().splitlines()
    assert out[-1] == "PRODUCT-NOT-LOADED"  # the reference arm runs none of this library's code
    line = json.loads(out[-2])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "evals/s" and line["higher_is_better"] is True
    assert line["steps"] == 1 and line["warmup"] == 0 and line["ms_per_step"] > 0
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "evals/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["photon_bins"] == 512 and line["config"]["particles"] == 99_000_000
