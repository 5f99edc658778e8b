"""CPU check of bench.py's output contract on its reference arm (the oracle
restatement timed on the host cores): one JSON line on stdout carrying every
key the harness reads, with consistent units and a zero-copy e2e block."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "768",
           "--nb", "64", "--nrhs", "2", "--steps", "1", "--warmup", "3"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["unit"] == "TFLOP/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["n"] == 768 and d["config"]["nb"] == 64 and d["config"]["nrhs"] == 2
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert cb["host_lapack"]["value"] > 0
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_phase_table_fractions():
    sys.path.insert(0, ROOT)
    import bench

    ph = {"laswp": (10, 5.0, 0.0, 4.0e9), "gemm": (4, 20.0, 8.0e12, 1.0e9), "solve": (0, 0.0, 0.0, 0.0)}
    t = bench.phase_table(ph, 2, 8000.0)
    assert set(t) == {"laswp", "gemm"}
    assert t["laswp"]["ms_per_step"] == 2.5 and t["laswp"]["tflops"] is None
    assert abs(t["laswp"]["gbs"] - 800.0) < 1e-9 and abs(t["laswp"]["hbm_frac"] - 0.1) < 1e-12
    assert abs(t["gemm"]["tflops"] - 400.0) < 1e-9
