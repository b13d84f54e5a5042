"""Host-side pieces of bench.py's output line, without a GPU: the FFT flop count, the traffic
figure read from the committed ncu summary, the workload table and the clock sampler's reading
of nvidia-smi lines (throttle reasons are what reject a measurement)."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fft_flop_count(bench):
    # three 2048-point t transforms and two each of the 256-point x and y transforms, 5 n log2 n
    assert bench.fft_flop_per_pt_step(256, 256, 2048) == pytest.approx(3 * 55 + 4 * 40)
    assert bench.fft_flop_per_pt_step(512, 512, 1024) == pytest.approx(3 * 50 + 4 * 45)


def test_profile_traffic_from_committed_summary(bench):
    algorithmic = 16 * 256 * 256 * 2048
    wl = bench.WORKLOADS["cell256"]["profile"]
    t = bench.profile_traffic(wl["pencil"])
    assert t is not None and 0.9 * algorithmic < t < 1.2 * algorithmic
    # the plane sweep's two kernels, summed: two passes over the field
    t2 = bench.profile_traffic(wl["plane"])
    assert t2 is not None and 1.8 * algorithmic < t2 < 2.4 * algorithmic
    assert bench.profile_traffic(["no_such_summary.txt"]) is None
    assert bench.profile_traffic(["pencil_step_256x256x2048.txt", "no_such_summary.txt"]) is None


def test_whole_run_accuracy_reader(bench, tmp_path, monkeypatch):
    class P:
        Nx, Ny, Nt = 8, 8, 16
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.whole_run_accuracy(P()) is None
    (tmp_path / "profiles").mkdir()
    (tmp_path / "profiles" / "accuracy_whole_run_8x8x16.txt").write_text(
        "command: x\nsplit_steps: 3200\nfield_rel_l2: 4.5e-05\nspectrum_rel_l2: 2e-05\nenergy_drift: 1e-6\n")
    r = bench.whole_run_accuracy(P())
    assert r["split_steps"] == 3200 and r["field_rel_l2"] == 4.5e-05 and r["energy_drift"] == 1e-6


def test_workloads_name_existing_cells(bench):
    from mpc_gb300 import inputs
    assert "cell256" in bench.WORKLOADS
    for name, wl in bench.WORKLOADS.items():
        cfg = getattr(inputs, wl["cell"])()
        assert cfg.Nx * cfg.Ny * cfg.Nt > 0 and wl["per_step"] > 0 and wl["cpu_steps"] > 0, name
    assert bench.WORKLOADS["cell512"]["adaptive"] and not bench.WORKLOADS["cell256"]["adaptive"]


def test_clock_sampler_reads_throttle_reasons(bench):
    s = bench.ClockSampler(0)
    s.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "garbage line"]

    class _Done:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    s.proc = _Done()
    out = s.stop()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"]
    s2 = bench.ClockSampler(0)
    s2.lines = ["0, 1200, 2070, 700.0, 0x8, Not Active, Active, Not Active, Not Active"]
    s2.proc = _Done()
    assert s2.stop()["reasons"] == ["hw_thermal_slowdown"]
