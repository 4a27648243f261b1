"""Host-side pieces of bench.py that need no GPU (CPU): the clock record
kept from nvidia-smi samples inside the timed windows, the DRAM traffic
figures read from the committed ncu summaries, and the compulsory bytes of
one 256^3 realisation."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _DoneProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def _sampler(lines, windows):
    s = bench.ClockSampler(0)
    s.proc = _DoneProc()
    s.lines = lines
    s.windows = windows
    return s


def test_clock_samples_inside_windows_only():
    ok = "2070, 2070, Not Active, Not Active, Not Active, Not Active"
    lines = [(0.5, "1000, 2070, Not Active, Not Active, Not Active, Not Active"),   # before: idle clock
             (1.5, ok), (1.7, ok),
             (2.5, "1500, 2070, Active, Not Active, Not Active, Not Active"),      # between the windows
             (3.2, "2070, 2070, Not Active, Not Active, Not Active, Active")]
    clk = _sampler(lines, [[1.0, 2.0], [3.0, 4.0]]).stop()
    assert clk["samples"] == 3
    assert clk["sm_mhz"] == 2070.0 and clk["sm_max_mhz"] == 2070.0
    assert clk["reasons"] == ["sw_power_cap"]      # hw_slowdown fell between the windows


def test_clock_window_without_sample_takes_the_one_before():
    lines = [(0.9, "2055, 2070, Not Active, Not Active, Not Active, Not Active"),
             (1.2, "2070, 2070, Not Active, Not Active, Not Active, Not Active")]
    clk = _sampler(lines, [[1.0, 1.05]]).stop()
    assert clk["samples"] == 1 and clk["sm_mhz"] == 2055.0


def test_clock_without_windows_uses_every_sample():
    lines = [(t, "2070, 2070, Not Active, Not Active, Not Active, Not Active") for t in (1.0, 2.0, 3.0)]
    assert _sampler(lines, []).stop()["samples"] == 3


def test_committed_traffic_covers_the_dominant_class():
    # the bench line's roofline names the strided FFT passes (the class with the most time); its traffic
    # comes from the committed ncu summary of one strided pass
    t = bench.committed_traffic()
    assert "fft_strided" in t and 1e6 < t["fft_strided"] < 2e8


def test_step_bytes_of_a_256_cube_realisation():
    # field 8Nc, c2r 8Nc + 4N, ladder 50 (8Nc + 2N), peaks + growth 8N, 1LPT 8Nc + 20N,
    # 2LPT 52N + 16Nc, CIC + P(k) 12 nh + 8N + 16Nc: about 7.09 GB with 1e6 halos
    b = bench.step_algorithmic_bytes(256, 50, 1.0e6)
    assert abs(b - 7.088e9) < 0.01e9


class _Range(RuntimeError):
    pass


def test_seed_policy_skips_range_errors_and_counts_completed_steps():
    def fn(s):
        if s in (3, 8):
            raise _Range()
        return s * 10

    out, done, skipped = bench.run_seeds(fn, 7, 1, _Range)
    assert done == [1, 2, 4, 5, 6, 7, 9] and skipped == [3, 8]
    assert out == [10, 20, 40, 50, 60, 70, 90]


def test_seed_policy_gives_up_after_many_range_errors():
    import pytest

    def fn(s):
        raise _Range()

    with pytest.raises(RuntimeError):
        bench.run_seeds(fn, 2, 1, _Range, max_skipped=3)


def test_reference_realisation_with_range_error_is_reported(orc, pk):
    """Seed 8 of the box_256 workload (taus field, barrier a=1 beta=0.12)
    grows a halo of ~5000 cells whose mass lies beyond the mass-function
    splines: the oracle raises its range error, which the benchmark's seed
    policy skips (the reference's GSL spline would abort)."""
    import pytest
    k, P = pk
    with pytest.raises(orc.RangeError):
        orc.halos_box_from_pk(k, P, nd=256, Lc=2.0, seed=8, stream=0, do_2lpt=0, prec="f32", a=1.0, beta=0.12,
                              alpha=0.0)
