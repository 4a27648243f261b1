"""Integer arithmetic the kernels use in place of slower forms, compiled as
plain C++ here (CPU):
- the CIC accumulator's fixed-point conversions (exshalos_gb300/csrc/
  fixedpoint.cuh) must give the bits of the FP64 expressions they restate:
  round(w 2^40) for every float w in [0, 1], and (float)((double)q 2^-40)
  for 2e7 sums q of every bit length, with ties at both rounding steps;
- the fast division of intdiv.cuh must equal x / d for 1.4e8 pairs (every
  d up to 5000, powers of two and their neighbours, random d; x at the ends
  of the range and next to multiples of d);
- the FP32 restatements of fp32sum.cuh: the 2LPT source combination within
  one float ulp of the FP64 form (and equal in all but a few of 2e7 cases,
  cancelling ones included), the compensated sum within 2^-23 of the total
  plus 2^-44 of the magnitudes."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run_check(tmp_path, name):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / name
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "exshalos_gb300", "csrc"),
                    os.path.join(ROOT, "tests", name + ".cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout


def test_fixedpoint_matches_fp64(tmp_path):
    _run_check(tmp_path, "fixedpoint_check")


def test_fastdiv_matches_division(tmp_path):
    _run_check(tmp_path, "intdiv_check")


def test_fp32_restatements_match_fp64(tmp_path):
    _run_check(tmp_path, "fp32sum_check")


def test_taus_draw_index_matches_the_reference_loop(tmp_path):
    _run_check(tmp_path, "taus_index_check")


def test_taus_chunked_polar_method_matches_sequential(tmp_path):
    _run_check(tmp_path, "taus_chunk_check")
