"""bench.py's reference arm (the reference's CPU algorithm, no GPU needed) prints one JSON line
with the keys the benchmark contract asks for."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--size", "256",
                          "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["workload"] == "ozaki_fp64_gemm_256^3"
    # the GPU arm prints the same config dict (its plan goes under a separate key)
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.headline_config(256, 256, 256, 1)
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


class _Ev:
    """A stand-in for a CUDA event: its time in ms from the window's start event."""

    def __init__(self, t):
        self.t = t

    def elapsed_time(self, other):
        return other.t - self.t


def test_pipeline_timeline_reports_stalls():
    """The end-to-end timeline of a ring of 4: uploads of 5 ms, computes of 10 ms, downloads of
    3 ms; step 6's upload takes 60 ms, so its compute waits for it.  The timeline names the
    wait, its length and the long upload, and counts every step's cause."""
    sys.path.insert(0, ROOT)
    import bench
    nbuf, steps = 4, 10
    up, comp, down = [], [], []
    up_end = [0.0] * steps
    comp_end = [0.0] * steps
    for i in range(steps):
        start = 0.0 if i == 0 else up_end[i - 1]
        if i >= nbuf:
            start = max(start, comp_end[i - nbuf])          # ring slot free once its compute ended
        length = 60.0 if i == 6 else 5.0
        up_end[i] = start + length
        up.append((_Ev(start), _Ev(up_end[i])))
        c0 = max(up_end[i], comp_end[i - 1] if i else 0.0)
        comp_end[i] = c0 + 10.0
        comp.append((_Ev(c0), _Ev(comp_end[i])))
        down.append((_Ev(comp_end[i]), _Ev(comp_end[i] + 3.0)))
    t = bench.pipeline_timeline(_Ev(0.0), up, comp, down, nbuf, [0.1 * i for i in range(steps)])
    assert t["upload_ms_max"] == 60.0
    stalls = {s["step"]: s for s in t["stalls"]}
    assert set(stalls) == {6}
    assert stalls[6]["waited_on"] == "upload" and stalls[6]["upload_ms"] == 60.0
    assert abs(stalls[6]["idle_ms"] - (up_end[6] - comp_end[5])) < 1e-9
    assert t["waited_on"]["upload"] == 2 and sum(t["waited_on"].values()) == steps
    assert abs(t["compute_idle_ms_total"] - (up_end[6] - comp_end[5])) < 1e-9
    assert len(t["steps"]) == 8
