"""The profiling driver's command line (CPU: argument parsing only; the
stages themselves need a GPU and run in the profile recipes)."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    return subprocess.run([sys.executable, "-m", "exshalos_gb300.profile_case", *args], cwd=ROOT,
                          capture_output=True, text=True, timeout=120)


def test_help_lists_the_stages():
    r = _run("--help")
    assert r.returncode == 0
    for stage in ("halos", "pk", "ladder", "fft", "grid512"):
        assert stage in r.stdout


@pytest.mark.parametrize("args", [("nope",), ()])
def test_unknown_or_missing_stage_is_refused(args):
    r = _run(*args)
    assert r.returncode != 0 and "usage" in r.stderr
