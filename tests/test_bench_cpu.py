"""Host-side pieces of bench.py that need no GPU: the clock-sample parsing, the
peak lookup, and the reference arm's JSON line (with a stand-in for the timed
CPU step)."""
import io
import json
import os
import sys
from contextlib import redirect_stdout

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def test_clock_samples_parsed():
    c = bench.ClockSampler(0)
    c.proc = _Done()
    c.skip = 1
    c.lines = ["0, 1500, 2070, 300.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 2070, 2070, 900.5, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2040, 2070, 950.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 2070, 2070, 940.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    got = c.stop()
    assert got == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_clock_sampler_without_samples():
    c = bench.ClockSampler(0)
    assert c.stop() is None


def test_measured_peak_fallback(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.measured_peak_hbm() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6798.9}))
    assert bench.measured_peak_hbm() == (6798.9, "measured")


class _FakePool:
    def close(self):
        pass

    def join(self):
        pass


def test_reference_arm_line(monkeypatch):
    """The reference arm's line carries the contract's keys, times full steps
    (``cpu_step``) after the warm-up ones, and stops timing at its budget (here:
    after the first timed step)."""
    import argparse
    calls = []

    def fake(pool, nproc, w, targets):
        calls.append((nproc, w, targets))
        return 20.0

    monkeypatch.setattr(bench, "reference_setup", lambda: (_FakePool(), 3, "w", "t"))
    monkeypatch.setattr(bench, "cpu_step", fake)
    monkeypatch.setattr(bench, "REFERENCE_BUDGET_S", -1.0)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_arm(argparse.Namespace(impl="reference", gpus=1, steps=400, warmup=2), 1, 0)
    line = json.loads(buf.getvalue().strip().splitlines()[-1])
    assert len(calls) == 3 and calls[0] == (3, "w", "t")
    assert line["impl"] == "reference" and line["steps"] == 400 and line["steps_timed"] == 1
    assert abs(line["value"] - 0.05) < 1e-12 and line["unit"] == "steps/s" and line["higher_is_better"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 3
    assert "full step" in line["cpu_baseline"]["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["timed_s"] == 20.0


def test_cpu_step_runs_the_oracle_step(monkeypatch):
    """cpu_step times one call of the oracle's full step on the given pool."""
    from oracle import parallel
    seen = []
    monkeypatch.setattr(parallel, "render_advect_step", lambda *a, **k: seen.append(a[:2]))

    class W:
        rho = ux = uy = uz = M = V = P = F = image_dhw = depth_step = None
    t = bench.cpu_step("pool", 7, W(), None)
    assert seen == [("pool", 7)] and t >= 0.0


def test_host_cpu_description(tmp_path):
    x86 = tmp_path / "x86"
    x86.write_text("processor\t: 0\nmodel name\t: Some CPU @ 2.0GHz\n\nprocessor\t: 1\n"
                   "model name\t: Some CPU @ 2.0GHz\n")
    assert bench.host_cpu(str(x86))["model"] == "Some CPU @ 2.0GHz"
    arm = tmp_path / "arm"
    arm.write_text("processor\t: 0\nCPU implementer\t: 0x41\nCPU part\t: 0xd4f\n\n"
                   "processor\t: 1\nCPU implementer\t: 0x41\nCPU part\t: 0xd4f\n")
    assert bench.host_cpu(str(arm))["model"] == "Neoverse-V2 (implementer 0x41)"
    other = tmp_path / "other"
    other.write_text("CPU implementer\t: 0x61\nCPU part\t: 0x022\n")
    assert bench.host_cpu(str(other))["model"] == "part 0x022 (implementer 0x61)"
    missing = bench.host_cpu(str(tmp_path / "absent"))
    assert "model" not in missing and missing["logical_cpus"] >= 1 and missing["arch"]
