"""Host-side logic of the benchmark that needs no GPU: the clock record taken
from nvidia-smi samples (which decides whether a run is kept) and the untimed
load phase that the samples are taken over."""
import importlib.util
import os
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_host_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class _Proc:
    """Stands in for the nvidia-smi process the sampler stops."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def _sampler_over(b, lines):
    s = b.ClockSampler(0)
    fd, path = tempfile.mkstemp(suffix=".csv")
    with os.fdopen(fd, "w") as f:
        f.write("\n".join(lines) + "\n")
    s.path = path
    s.fh = open(os.devnull, "w")
    s.proc = _Proc()
    return s, path


def test_clock_record_median_and_reasons():
    b = load_bench()
    na = "Not Active"
    s, path = _sampler_over(b, [
        f"0, 2070, 2070, 910.2, 0x0000000000000000, {na}, {na}, {na}, {na}",
        f"0, 1980, 2070, 1390.0, 0x0000000000000004, {na}, {na}, {na}, Active",
        f"0, 2070, 2070, 1200.5, 0x0000000000000000, {na}, {na}, {na}, {na}",
        "garbage line",
    ])
    rec = s.stop()
    assert not os.path.exists(path)      # the temporary CSV is removed
    assert rec["samples"] == 3           # malformed lines are skipped
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["reasons"] == ["sw_power_cap"]


def test_clock_record_names_every_slowdown_reason():
    b = load_bench()
    s, _ = _sampler_over(b, ["0, 1500, 2070, 1400.0, 0x00000000000000e8, Active, Active, Active, Active"])
    rec = s.stop()
    assert rec["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap", "sw_thermal_slowdown"]
    assert rec["sm_mhz"] == 1500.0


def test_clock_record_without_samples_or_sampler():
    b = load_bench()
    s, _ = _sampler_over(b, [])
    assert s.stop() is None
    assert b.ClockSampler(0).stop() is None   # nvidia-smi never started
    assert b.with_window(None) is None
    assert "window" in b.with_window({"samples": 1})


def test_load_phase_runs_steps_for_the_given_time(monkeypatch):
    torch = pytest.importorskip("torch")
    b = load_bench()
    syncs = []
    monkeypatch.setattr(torch.cuda, "synchronize", lambda device=None: syncs.append(device))
    steps = []
    b.load_phase(lambda i: steps.append(i), "cuda:0", seconds=0.05)
    assert steps == list(range(len(steps))) and len(steps) >= 16 and len(steps) % 16 == 0
    assert syncs and all(d == "cuda:0" for d in syncs)


def test_f2x3_report_records_a_failing_path_instead_of_raising():
    """A failure of either F(2x3) path is reported in the bench line; the
    headline it sits beside is not lost."""
    b = load_bench()

    class _Buf:
        def data_ptr(self):
            return 16

    class _Err(Exception):
        pass

    class _Wg:
        ALGO_2X3, ALGO_2X3_FUSED = 1, 2

        @staticmethod
        def make_problem(*a):
            return a

        @staticmethod
        def default_options(algo):
            return algo

        @staticmethod
        def Conv2d(prob, opts):
            raise _Err(f"cannot plan algorithm {opts}")

    out = b.f2x3_paths(_Wg, None, [_Buf()], [_Buf()], _Buf(), (1, 8, 8, 8, 8), 0, "cuda:0", 3,
                       {"hbm_gbs": 1.0, "bf16_tflops": 1.0}, "measured")
    assert set(out) == {"non_fused", "fused"}
    assert out["non_fused"]["error"] == "_Err: cannot plan algorithm 1"
    assert out["fused"]["error"] == "_Err: cannot plan algorithm 2"


def test_algorithmic_and_design_bytes():
    """The roofline counts V + U for the GEMM and y for the output transform
    (M excluded); the design bytes add M, 24-bit M padded to blocks of 64
    tiles (N32 C512 28x28 K512: 1568 tiles -> 1600), fp32 and fp16 M not."""
    b = load_bench()
    E = 36
    # N32 C256 56x56 K256, F(4x3): 6272 tiles, a multiple of 64
    alg, design, flops, _ = b.algorithmic_work("gemm_tcgen05", (32, 256, 56, 56, 256, 4))
    v, u, m = 2.0 * E * 6272 * 256, 2.0 * E * 256 * 256, 3.0 * E * 6272 * 256
    assert alg == pytest.approx(v + u) and design == pytest.approx(v + u + m)
    assert flops == pytest.approx(2.0 * E * 6272 * 256 * 256)
    # N32 C512 28x28 K512: 1568 tiles, 24-bit M over 1600
    alg, design, _, _ = b.algorithmic_work("output_transform", (32, 512, 28, 28, 512, 4))
    y = 2.0 * 32 * 512 * 28 * 28
    assert alg == pytest.approx(y) and design == pytest.approx(y + 3.0 * E * 1600 * 512)
    # fp32 M is not padded
    _, design, _, _ = b.algorithmic_work("output_transform", (32, 512, 28, 28, 512, 4), 4.0)
    assert design == pytest.approx(y + 4.0 * E * 1568 * 512)
