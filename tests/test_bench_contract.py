"""bench.py's reference arm on the CPU: the JSON line's contract (keys,
units, the bounded sample it describes, a step time that is the step it
timed), on a shrunken workload so that it runs in seconds; and that the arm
neither imports the product package nor loads its library."""
import json
import pathlib
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent

RUNNER = """
import runpy, sys
sys.argv = {argv!r}
runpy.run_path({bench!r}, run_name="__main__")
maps = open("/proc/self/maps").read() if sys.platform.startswith("linux") else ""
print("PRODUCT", any(m == "pypo_gb300" or m.startswith("pypo_gb300.") for m in sys.modules),
      "libpo_gb300" in maps)
"""


@pytest.mark.parametrize("workload", ["dish_eh", "dish_chain"])
def test_reference_arm_line(workload):
    argv = ["bench.py", "--impl", "reference", "--workload", workload, "--steps", "2", "--scale", "0.05",
            "--cpu-seconds", "3"]
    code = RUNNER.format(argv=argv, bench=str(ROOT / "bench.py"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["impl"] == "reference" and line["unit"] == "Gpairs/s" and line["value"] > 0
    assert line["warmup"] >= 3 and line["steps"] == 2 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"] and cb["value"] == line["value"]
    assert "forward + adjoint" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "Gpairs/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cfg = line["config"]
    assert cfg["workload"].startswith(workload) and "adjoint" in cfg["step"] + cfg["step"].replace("backward", "adjoint")
    assert set(cfg) >= {"workload", "desc", "pairs_per_step", "step", "l2"}
    # the step time is the sampled step as timed: value = timed pairs / step time
    timed = line["value"] * 1e9 * line["ms_per_step"] * 1e-3
    assert abs(timed - line["timed_pairs_per_step"]) <= 1e-6 * line["timed_pairs_per_step"]
    assert line["timed_pairs_per_step"] <= cfg["pairs_per_step"]
    # no product code on this arm
    flags = [ln for ln in r.stdout.splitlines() if ln.startswith("PRODUCT")][-1].split()
    assert flags[1:] == ["False", "False"], flags
