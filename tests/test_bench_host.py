"""Host logic of bench.py, on CPU: the clock record parsed from nvidia-smi's CSV lines, the
measured-peak lookup, the illumination tilts of the batched workload, and the JSON line of
the reference arm (its CPU sample replaced by a fixed figure, so the test takes no time)."""
import argparse
import importlib.util
import json
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_summary(bench):
    c = bench.ClockSampler(0)
    na = "Not Active"
    c.lines = [
        "0, 2070, 2070, 901.5, 0x0000000000000000, %s, %s, %s, %s" % (na, na, na, na),
        "0, 1980, 2070, 1391.0, 0x0000000000000004, %s, %s, %s, Active" % (na, na, na),
        "0, 2070, 2070, 1010.2, 0x0000000000000000, %s, %s, %s, %s" % (na, na, na, na),
        "0, [N/A], 2070, 0, 0x0, %s, %s, %s, %s" % (na, na, na, na),   # unreadable clock: skipped
        "No devices were found",                                       # not a sample line
    ]
    assert c.summary() == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"],
                           "samples": 3}
    c.lines = ["0, 1500, 2070, 700, 0x0, Active, %s, Active, %s" % (na, na)]
    s = c.summary()
    assert s["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"] and s["sm_mhz"] == 1500.0
    c.lines = []
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_clock_sampler_returns(bench):
    # without a GPU, nvidia-smi is absent or exits at once: the sampler neither raises nor waits
    # longer than its start-up limit, and records no sample line; with one it records samples
    import time
    t0 = time.time()
    with bench.ClockSampler(0) as c:
        pass
    assert time.time() - t0 < 15
    s = c.summary()
    assert (s["samples"] == 0) == (s["sm_mhz"] is None)


def test_peaks_read_the_measured_file(bench):
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    gbs, kind = bench.peaks()
    if os.path.exists(p):
        assert kind == "measured" and gbs == float(json.load(open(p))["hbm_gbs"])
    else:
        assert kind == "fallback" and gbs == 6800.


def test_fp32_peak_formula(bench):
    # 152 SMs x 128 FP32 lanes x 2 flops x clock
    assert bench.fp32_peak_tflops(2070.) == pytest.approx(152 * 128 * 2 * 2.07e9 / 1e12)


def test_tilts_inside_the_aperture(bench):
    u0 = bench.make_u0(64, 32, 16, bench.SEED + 1)
    assert u0.shape == (64, 16, 32) and u0.dtype == np.complex64
    assert np.allclose(np.abs(u0), 1, atol=1e-6)
    k0 = 2 * np.pi / bench.LAM
    # plane waves exp(-i(kx x + ky y)): the phase step of one pixel gives the tilt (|k dx| < pi)
    kx = -np.angle(u0[:, 0, 1] / u0[:, 0, 0]) / bench.UNITS[0]
    ky = -np.angle(u0[:, 1, 0] / u0[:, 0, 0]) / bench.UNITS[1]
    na = np.hypot(kx, ky) / k0
    assert na.max() <= .8 + 1e-5
    # area-uniform in the disk: about a quarter of the tilts fall inside radius 0.4
    assert 6 <= int((na < .4).sum()) <= 28
    assert np.array_equal(u0, bench.make_u0(64, 32, 16, bench.SEED + 1))


def test_reference_arm_line(bench, monkeypatch):
    calls = []

    def fake_sample(fields=1, steps=48):
        calls.append((fields, steps))
        return 2.5e7, .05, "%d field(s) x 512x512 x %d z-steps" % (fields, steps)

    monkeypatch.setattr(bench, "cpu_sample", fake_sample)
    args = argparse.Namespace(warmup=3, steps=4)
    assert bench.bench_reference(args, 1) is None and calls == []
    line = bench.bench_reference(args, 0)
    assert len(calls) == 7
    json.dumps(line)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["config"]["workload"] == bench.WORKLOAD
    assert line["value"] == 2.5e7 and line["ms_per_step"] == pytest.approx(50.)
    assert line["higher_is_better"] is True and line["vs_baseline"] is None
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"] == {"value": 2.5e7, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_gpus_flag_launches_the_ranks():
    """bench.py --gpus 2 with no external launcher starts two ranks itself (one process each,
    rendezvous on 127.0.0.1); --check-launch makes every rank join a gloo group and rank 0
    report how many arrived, with no GPU work."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--check-launch"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    assert json.loads(lines[0]) == {"check_launch": True, "ranks": 2, "world_size": 2}
