"""bench.py on the CPU: the reference arm's JSON line (it times the oracle restatement of the
reference's update loop and needs no GPU) and the workload definitions."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("config", ["c1", "c4"])
def test_reference_arm_prints_its_line(config):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", config, "--steps", "3",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "spin updates/s" and line["unit"] == "updates/s" and line["higher_is_better"]
    assert line["value"] > 0 and line["steps"] == 3 and line["warmup"] == 3
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "updates/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_workloads_have_the_documented_sizes():
    sys.path.insert(0, ROOT)
    import bench

    c4 = bench.make_config("c4")
    assert (c4["shape"], c4["edge"], len(c4["T"]), c4["periodic"], c4["D"], c4["samp"]) == ("c", 128, 40, True, 0.3, 10)
    assert c4["bytes_per_update"] == 36 and min(c4["T"]) == 0.2 and max(c4["T"]) == 2.0
    c1 = bench.make_config("c1")
    assert (c1["shape"], c1["edge"], len(c1["T"]), c1["ising"], c1["bytes_per_update"]) == ("s", 32, 13, True, 3)
    c2 = bench.make_config("c2")
    assert (c2["shape"], c2["edge"], len(c2["T"]), c2["D"], c2["samp"]) == ("s", 64, 420, 0.5, 20)
    c3 = bench.make_config("c3")
    assert (c3["shape"], c3["edge"], len(c3["T"]), c3["amean"], c3["asd"]) == ("w", 90, 512, 20.0, 5.0)
    x3 = bench.make_config("x3")
    assert (x3["shape"], x3["edge"], len(x3["T"]), x3["amean"]) == ("x", 90, 96, 30.0)
    j2 = bench.make_config("c4j2")
    assert (j2["shape"], j2["edge"], len(j2["T"]), j2["jfile"]) == ("c", 128, 40, "3d_j1j2_bloch.dat")
    with pytest.raises(ValueError):
        bench.make_config("c9")
