"""Host-side pieces of bench.py on the CPU: the clock sampler's summary (the
samples inside the timed window, throttle reasons), the roofline figures
from per-call records, and the per-pass reductions with one rank."""
import datetime
import os
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _clock_rows(t0, n, period, active_at=()):
    rows = []
    for i in range(n):
        ts = datetime.datetime.fromtimestamp(t0 + i * period).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        cap = "Active" if i in active_at else "Not Active"
        rows.append(f"{ts}, 0, {2070 - i}, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, {cap}")
    return rows


def test_clock_summary_keeps_the_timed_window():
    c = bench.Clocks(0)
    c.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    now = time.time()
    c.f.write("\n".join(_clock_rows(now, 20, 0.1, active_at=(15,))) + "\n")
    c.window = [now + 0.475, now + 1.075]    # samples 5 .. 11 (with the 50 ms margin)
    s = c.summary()
    assert s["window"] == "timed steps"
    assert s["samples"] == 7
    assert s["sm_mhz"] == 2070 - 8
    assert s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == []               # the power-cap sample lies outside the window


def test_clock_summary_falls_back_to_every_sample():
    c = bench.Clocks(0)
    c.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
    now = time.time()
    c.f.write("\n".join(_clock_rows(now, 5, 0.1, active_at=(2,))) + "\n")
    c.window = [now + 10.0, now + 10.1]      # nothing inside
    s = c.summary()
    assert s["window"] == "warm-up and timed steps" and s["samples"] == 5
    assert s["reasons"] == ["sw_power_cap"]


def test_roofline_from_call_records():
    u = dict(n=1000, od=65, evals=13, active=16, levels=16, tbytes=4, train=True)
    summary = {"angelo_sdf_stencil_bwd": (2, 4.0, [u, u]), "angelo_adamw_step": (2, 1.0, [dict(n=10)] * 2)}
    rl, shares = bench.roofline(summary, 6000.0, "measured")
    per = bench.algorithmic_bytes("angelo_sdf_stencil_bwd", u)
    assert rl["kernel"] == "angelo_sdf_stencil_bwd" and rl["launches"] == 2
    assert rl["bytes_per_launch"] == per
    assert abs(rl["achieved"] - 2 * per / 4e-3 / 1e9) < 0.1
    assert abs(rl["frac"] - rl["achieved"] / 6000.0) < 1e-4
    assert rl["traffic"] == int(bench.TRAFFIC_BYTES_PER_SAMPLE["angelo_sdf_stencil_bwd"] * 1000)
    assert list(shares) == ["angelo_sdf_stencil_bwd", "angelo_adamw_step"]


def test_dynamic_ray_count_targets_and_counts_the_background():
    """The learned-background form aims its dynamic ray count at the
    reference's target with the background's samples
    (train_num_rays * (num_samples_per_ray + num_samples_per_ray_bg),
    systems/neus.py:28), and the count compared with it is the foreground's
    plus the kept background samples (num_samples_full)."""
    import torch
    _, tr = bench.make_trainer("fused", torch.device("cpu"))
    assert tr.train_num_samples == 1 << 18
    m, tr = bench.make_trainer("fused_bg", torch.device("cpu"))
    assert tr.train_num_samples == (1 << 18) * (512 + 256) // 512
    assert m.last_num_samples is None
    m._n_fg, m._n_bg = 1000, 250
    assert m.last_num_samples == 1250
