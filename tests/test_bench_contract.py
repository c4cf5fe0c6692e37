"""bench.py's reference arm (the CPU implementation of the step on the host
cores) prints one JSON line with the metric, unit and config of the GPU
arm, a cpu_baseline block describing the run, and an e2e block with no
host-device bytes.  Runs on CPU, on a small workload."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    env = dict(os.environ, CYLAG_REF_SAMPLE="2000")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--steps", "2", "--warmup", "1", "--npart", "5000", "--nx", "101",
                        "--ny", "26"], capture_output=True, text=True, env=env, timeout=600,
                       cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("particle-steps/s")
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["config"]["workload"].startswith("lsm1_2d")
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference")
    assert cb["cores"] >= 1 and "2000" in cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_lsm1_workload_records_cover_the_horizon():
    """The k-eps drift workload's field records: A, B, A at 0 / 600 / 1200 s
    by default, continued A, B, ... every 600 s for longer horizons, so that
    warm-up, timed and end-to-end steps never extrapolate in time."""
    import numpy as np
    from cylag_gb300 import synth
    a = synth.keps_drift_channel(npart=10, nx=21, ny=6, seed=0)
    np.testing.assert_array_equal(a["times"], [0.0, 600.0, 1200.0])
    b = synth.keps_drift_channel(npart=10, nx=21, ny=6, seed=0, horizon=3000.0)
    np.testing.assert_array_equal(b["times"], 600.0 * np.arange(6))
    np.testing.assert_array_equal(b["velocity_x"][:3], a["velocity_x"])
    for r in range(6):
        np.testing.assert_array_equal(b["velocity_x"][r], a["velocity_x"][r % 2])
        np.testing.assert_array_equal(b["opt_fields"][:, r], a["opt_fields"][:, 0])


def test_clock_record_parsing():
    """The clocks block of a bench line: median SM clock under load, the
    maximum, and every throttle reason seen active during the timed region."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    class Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    cs = bench.ClockSampler(0)
    cs.proc = Done()
    cs.lines = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1320.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbled",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    got = cs.stop()
    assert got["sm_mhz"] == 2070.0 and got["sm_max_mhz"] == 2070.0
    assert got["reasons"] == ["sw_power_cap"] and got["samples"] == 3
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]
