"""Host logic of the benchmark driver (no GPU): the clock and throttle-reason parsing of the
nvidia-smi sampler, the per-kernel roofline selection, and the single-rank replica arithmetic."""
import json
import os

import pytest

import bench


class _FakeProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _clocks_from_rows(rows):
    c = bench.Clocks(None)
    c.f.write("\n".join(rows) + "\n")
    c.p = _FakeProc()   # as if the sampler had run
    return c.stop()


def test_clocks_median_and_reasons():
    # index, bus, sm MHz, max MHz, power, active mask, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    rows = ["0, 00000000:07:00.0, 2070, 2070, 612.3, 0x0000, Not Active, Not Active, Not Active, Not Active",
            "0, 00000000:07:00.0, 1965, 2070, 1390.1, 0x0004, Not Active, Not Active, Not Active, Active",
            "0, 00000000:07:00.0, 2070, 2070, 700.0, 0x0000, Not Active, Not Active, Not Active, Not Active"]
    r = _clocks_from_rows(rows)
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0
    assert r["power_w_max"] == pytest.approx(1390.1)
    assert r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]


def test_clocks_thermal_reasons_and_bad_rows():
    rows = ["0, x, 1500, 2070, 900, 0x0040, Active, Not Active, Active, Not Active",
            "garbage line",
            "0, x, [N/A], 2070, 900, 0x0, Not Active, Not Active, Not Active, Not Active"]
    r = _clocks_from_rows(rows)
    assert r["samples"] == 1 and r["sm_mhz"] == 1500.0
    assert r["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_clocks_without_samples_or_sampler():
    assert _clocks_from_rows([""])["reasons"] == ["no samples"]
    c = bench.Clocks(None)
    os.unlink(c.f.name)
    assert c.stop()["reasons"] == ["nvidia-smi unavailable"]


class _FakeLib:
    def __init__(self, prof):
        self.prof = prof
        self.enabled = []

    def prof_enable(self, on):
        self.enabled.append(on)

    def prof_read_all(self):
        return self.prof


class _FakeF:
    def __init__(self, prof):
        self._lib = _FakeLib(prof)


def test_prof_roofline_dominant_kernel():
    prof = {"s2s_xmix": (40.0, 9.6e10, 4), "s2s_yinv": (22.0, 7.0e10, 4), "bin": (1.0, 1.0e9, 1)}
    F = _FakeF(prof)
    calls = []
    r = bench.prof_roofline(F, lambda: calls.append("run"), lambda: calls.append("sync"))
    assert calls == ["run", "sync"] and F._lib.enabled == [True, False]
    peak, _ = bench.read_peaks()
    assert r["kernel"] == "s2s_xmix"
    assert r["achieved"] == pytest.approx(9.6e10 / 0.040 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    assert r["launches_per_step"] == 4 and r["avg_launch_ms"] == pytest.approx(10.0)
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(2.4e10)
    assert r["share_of_step"] == pytest.approx(40.0 / 63.0)
    assert list(r["all_kernels"]) == ["s2s_xmix", "s2s_yinv", "bin"]
    assert r["step_alg_bytes_GB"] == pytest.approx((9.6e10 + 7.0e10 + 1.0e9) / 1e9)
    json.dumps(r)   # the line stays serialisable
    assert bench.prof_roofline(_FakeF({}), lambda: None, lambda: None) is None


def test_peaks_read_from_the_measured_file():
    peak, kind = bench.read_peaks()
    bf16, bkind = bench.read_bf16_peak()
    if os.path.exists(os.path.join(bench.ROOT, "MEASURED_PEAKS.json")):
        assert kind == "measured" and bkind.startswith("measured")
        d = json.load(open(os.path.join(bench.ROOT, "MEASURED_PEAKS.json")))
        assert peak == float(d["hbm_gbs"]) and bf16 == float(d["bf16_tflops"])
    else:
        assert (peak, bf16) == (bench.FALLBACK_HBM_GBS, bench.FALLBACK_BF16_TFLOPS)


def test_single_rank_replica_arithmetic():
    assert bench.allmax(1, 3.5) == 3.5
    value, ms = bench.replica_throughput(1, 1.0, 91.5)
    assert ms == 91.5 and value == pytest.approx(1000.0 / 91.5)


def test_default_arguments_meet_the_contract(monkeypatch):
    """No flags: one GPU, the 512^3 headline configuration, at least 3 warm-up steps, our arm; every
    config the dispatcher knows is accepted by the parser."""
    import sys
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.config == "s2s" and a.impl == "ours" and a.n == 512
    assert a.warmup >= 3 and a.steps >= 1
    src = open(os.path.join(bench.ROOT, "bench.py")).read()
    import re
    for cfg in re.findall(r'args\.config == "([a-z0-9]+)"', src) + ["xpass", "ypass", "zbin"]:
        monkeypatch.setattr(sys, "argv", ["bench.py", "--config", cfg])
        assert bench.parse().config == cfg


def test_fused_pass_hook_rejects_bad_arguments():
    """The single-kernel benchmark hook validates its arguments before touching a GPU."""
    import ctypes as C
    import fit_gb300 as F
    lib = F._lib.load()
    ms, by = C.c_double(), C.c_double()
    for args in ((3, 512, 1, 1), (2, 512, 9, 1), (2, 512, 0, 1), (0, 512, 17, 1), (1, 512, 513, 1),
                 (1, 100, 1, 1), (0, 512, 16, 0)):
        assert lib.fit_bench_fused_pass(*args, C.byref(ms), C.byref(by)) == -1, args
