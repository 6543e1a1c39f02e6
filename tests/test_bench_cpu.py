"""bench.py's reference arm runs on the host cores alone (the oracle port of
the reference's likelihood path) and prints the contract's JSON line."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
           "--families", "300"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["unit"] == "family-lnL evals/s" and line["dtype"] == "f64"
    assert line["config"]["workload"].startswith("config1_gamma_k4_24taxa")
    base = line["cpu_baseline"]
    assert base["kind"] in ("port", "reference") and base["cores"] >= 1 and base["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_maps_only_the_oracle():
    """The timed reference arm must not run any of the product: after a run,
    the process has mapped the oracle's library and not libcafe_gb300.so
    (the workload's gamma multipliers come from the oracle's get_gamma)."""
    code = ("import sys, bench; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', "
            "'--families', '200', '--candidates', '2']; bench.main(); maps = open('/proc/self/maps').read(); "
            "print('product=%d oracle=%d' % ('libcafe_gb300' in maps, 'libcafe_oracle' in maps))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.strip().splitlines()
    line = json.loads(out[-2])
    assert line["config"]["candidates_per_step"] == 2 and line["config"]["families_per_gpu"] == 200
    assert out[-1] == "product=0 oracle=1", out[-1]
