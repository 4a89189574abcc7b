"""Host-side logic of the measurement tools, on the CPU: the benchmark's clock record (the
rule that rejects a throttled run reads it), its DRAM-traffic scaling from the committed
ncu capture, and the QRCP launch-choice report."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Done:
    """Stands in for the finished nvidia-smi process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _sampler(bench, tmp_path, lines):
    path = tmp_path / "clocks.csv"
    path.write_text("\n".join(lines) + "\n")
    s = bench.ClockSampler(0)
    s.proc = _Done()
    s.path = str(path)
    return s


def test_clock_record_median_and_reasons(tmp_path):
    bench = _bench()
    # index, sm, max sm, power, active mask, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    lines = [
        "0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    rec = _sampler(bench, tmp_path, lines).stop()
    assert rec["samples"] == 3
    assert rec["sm_mhz"] == 2070.0
    assert rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"]


def test_clock_record_flags_thermal_slowdown(tmp_path):
    bench = _bench()
    lines = [
        "0, 1500, 2070, 1400.0, 0x40, Not Active, Active, Not Active, Not Active",
        "0, 1490, 2070, 1400.0, 0x40, Active, Active, Not Active, Not Active",
    ]
    rec = _sampler(bench, tmp_path, lines).stop()
    assert rec["sm_mhz"] == pytest.approx(1495.0)
    assert rec["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"]


def test_clock_record_without_samples(tmp_path):
    bench = _bench()
    rec = _sampler(bench, tmp_path, []).stop()
    assert rec["sm_mhz"] is None and rec["reasons"] == ["no samples"]
    s = bench.ClockSampler(0)  # never started
    assert s.stop()["reasons"] == ["nvidia-smi unavailable"]


def test_traffic_scaled_from_committed_capture():
    bench = _bench()
    # the QRCP's DRAM-to-algorithmic ratio comes from its committed 32^3 capture
    assert bench.ncu_traffic("qrcp", 1.0e6) == round(0.62 * 1.0e6)
    assert bench.ncu_traffic("no_such_kernel", 1.0e6) is None


def test_tune_report_counts_and_ratio():
    from spand_public_gb300 import tune_report as tr

    rows = [
        dict(key="L0w0", items=10, cap=32, tuned="1x256s", tuned_ms=1.00, best="1x256s", best_ms=1.00, nforced=4,
             timed=[("1x256s", 0.99), ("2x128s", 1.10)]),
        dict(key="L0w1", items=10, cap=32, tuned="2x128s", tuned_ms=1.10, best="1x256s", best_ms=1.00, nforced=4,
             timed=[]),
        dict(key="L1w0", items=3, cap=64, tuned="4x256v", tuned_ms=0.50, best=None, best_ms=float("nan"),
             nforced=0, timed=[]),
    ]
    text = tr.report(rows, 64, 12, 1e-2, True, 3)
    assert "waves compared: 2 of 3" in text
    assert "tuned within 2% of the best forced: 1" in text
    assert "sum tuned 2.100 ms, sum best forced 2.000 ms (ratio 1.050)" in text
    assert "largest ratio: L0w1 1.100" in text
    assert "| L0w0 | 10 | 32 | 1x256s | 1.0000 | 1x256s | 1.0000 | 1.000 | 4 | 1x256s 0.990, 2x128s 1.100 |" in text
    assert "| L1w0 | 3 | 64 | 4x256v | 0.5000 | - |" in text
