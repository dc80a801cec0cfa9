"""Host-side pieces of bench.py, on the CPU.

The clock sampler's window logic is checked against a stand-in nvidia-smi that prints one
sample every 20 ms. The algorithmic bytes per particle are checked against their
definition: 4 n̄ + 24 for pass A, 4 n̄ + 44 for pass B and 24 n̄ + 352 for the step.
"""
import os
import time

import pytest

import bench

IDLE = "2070, 2070, Not Active, Not Active, Not Active, Not Active"


def _fake_smi(tmp_path, line, delay=0.2):
    p = tmp_path / "nvidia-smi"
    p.write_text(f'#!/bin/bash\nsleep {delay}\nwhile true; do echo "{line}"; sleep 0.02; done\n')
    p.chmod(0o755)
    return str(tmp_path) + os.pathsep + os.environ.get("PATH", "")


def test_clock_sampler_keeps_the_samples_of_the_region(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, IDLE))
    with bench.ClockSampler(0) as c:
        time.sleep(0.25)
    s = c.summary()
    assert s["window"] == "timed region"
    assert s["samples"] >= 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == []


def test_clock_sampler_reports_throttle_reasons(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, "1500, 2070, Not Active, Active, Not Active, Active"))
    with bench.ClockSampler(0) as c:
        time.sleep(0.1)
    s = c.summary()
    assert s["sm_mhz"] == 1500.0
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_short_region_takes_the_next_sample(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", _fake_smi(tmp_path, IDLE))
    with bench.ClockSampler(0) as c:
        pass
    s = c.summary()
    assert s["samples"] == 1
    assert s["window"] in ("timed region", "first sample after the timed region")


def test_no_nvidia_smi_means_unsampled(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))
    with bench.ClockSampler(0) as c:
        pass
    assert c.summary()["reasons"] == ["unsampled"]


@pytest.mark.parametrize("nbar", [1.0, 48.94, 60.0])
def test_algorithmic_bytes(nbar):
    ab = bench.algorithmic_bytes(nbar)
    assert ab["pass_a"] == pytest.approx(4 * nbar + 24)
    assert ab["pass_b"] == pytest.approx(4 * nbar + 44)
    assert ab["step"] == pytest.approx(24 * nbar + 352)


def _args(**kw):
    import argparse
    a = dict(gpus=2, steps=1, warmup=0, impl="reference", workload="dambreak_dx1024", no_cpu_baseline=True)
    a.update(kw)
    return argparse.Namespace(**a)


def test_reference_arm_prints_only_on_rank_zero(monkeypatch, capsys):
    """Under torchrun the reference arm runs on rank 0 alone; the other ranks exit without
    work and print nothing."""
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(_args())
    assert capsys.readouterr().out == ""


@pytest.mark.parametrize("workload", ["learned_fourier_b32", "adjoint_fourier128"])
def test_reference_arm_without_a_reference_path_says_why(monkeypatch, capsys, workload):
    import json
    monkeypatch.setenv("RANK", "0")
    bench.run_reference(_args(workload=workload))
    line = json.loads(capsys.readouterr().out.strip())
    assert line["impl"] == "reference" and line["unavailable"]


def test_reference_arm_outlet_step_matches_the_reference():
    """The host step that the mirror-outlet workload's reference arm and CPU baseline time
    (bench.regions_oracle_step) against the reference's own outlet update on the same block
    (tests/golden/make_outlet_step_golden.py): same ghosts, densities and velocities within
    1e-6 of their magnitudes (the consistent interpolation's rounding)."""
    import numpy as np
    from golden_io import GOLDEN, rel_max
    z = np.load(os.path.join(GOLDEN, "outlet_step_block32.npz"))
    fl = {k.split("/")[-1]: z[k].copy() for k in z.files if k.startswith("in/fluid/")}
    _, cfg = bench._regions_block(32, 0.9)
    assert bench.regions_oracle_step(fl, cfg, 0.9) == int(z["out/ghosts"])
    assert rel_max(fl["densities"], z["out/densities"]) < 1e-6
    assert rel_max(fl["velocities"], z["out/velocities"]) < 1e-6
    assert not np.array_equal(z["out/densities"], z["in/fluid/densities"])


def test_reference_arm_of_the_mirror_outlet(monkeypatch, capsys):
    """The mirror-outlet workload's reference arm: one oracle process per host core on the
    128^2 sample, in the workload's own unit."""
    import json
    monkeypatch.setenv("RANK", "0")
    bench.run_reference(_args(workload="outlet_mirror_1024", steps=1, warmup=0))
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "ghost-updates/s"
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["metric"] == bench.REGIONS_METRIC
