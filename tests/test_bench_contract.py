"""The benchmark's contract on the host, without a GPU: the reference arm's
JSON line (the CPU restatement timed on the host cores on a bounded sample),
the same arm under torchrun with two ranks (rank 0 alone prints, the other
rank exits 0 without work), the roofline denominator read from the measured
peaks, and the clock record parsed from nvidia-smi's CSV samples."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def _json_lines(text):
    return [json.loads(ln) for ln in text.splitlines() if ln.startswith("{")]


def _check_reference_line(d, steps, warmup, n_gpus):
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["steps"] == steps and d["warmup"] == warmup and d["n_gpus"] == n_gpus
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["dtype"] == "f64" and d["data"] == "synthetic"
    assert "workload" in d["config"] and "arm" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("port", "reference") and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_line():
    env = dict(os.environ, OMP_NUM_THREADS="4")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    _check_reference_line(lines[0], 1, 3, 1)
    assert lines[0]["cpu_baseline"]["cores"] == 4


def test_reference_arm_two_ranks():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    _check_reference_line(lines[0], 1, 3, 2)


def test_measured_peak_is_the_denominator():
    peak, kind = bench.measured_peak_hbm()
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        assert kind == "measured" and peak == float(json.loads(p.read_text())["hbm_gbs"])
    else:
        assert (peak, kind) == (6800.0, "fallback")


class _Proc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


class _Thread:
    def join(self, timeout=None):
        pass


def test_clock_record_from_samples():
    cs = bench.ClockSampler(0)
    cs.proc, cs.t = _Proc(), _Thread()
    row = "0, {sm}, 2070, 900.0, 0x0, {hw}, Not Active, Not Active, {pc}"
    cs.lines = [row.format(sm=2070, hw="Not Active", pc="Not Active"),
                row.format(sm=2055, hw="Not Active", pc="Active"),
                row.format(sm=2070, hw="Not Active", pc="Not Active"),
                "garbled line"]
    rec = cs.stop()
    assert rec["sm_mhz"] == 2070 and rec["sm_max_mhz"] == 2070 and rec["samples"] == 3
    assert rec["reasons"] == ["sw_power_cap"]
    cs = bench.ClockSampler(0)
    cs.proc, cs.t = _Proc(), _Thread()
    cs.lines = [row.format(sm=1500, hw="Active", pc="Not Active")]
    assert bench.ClockSampler.stop(cs)["reasons"] == ["hw_slowdown"]
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]
