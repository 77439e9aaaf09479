"""The smoothers' division by 6 (div6_rn in flub_gb300/csrc/smooth8.cuh):
Markstein's FMA correction must equal IEEE single-precision a / 6 for every
float32 in the range the kernels send through it.  Compiled and run on the
host (gcc, OpenMP), about a minute of CPU on 8 cores."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_div6_matches_ieee_division_for_every_float_in_range():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "div6_check")
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-o", exe,
                        os.path.join(HERE, "native", "div6_check.c"), "-lm"], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, timeout=1200)
    assert out.returncode == 0, out.stdout + out.stderr
    checked, bad = (int(x.split()[-1]) for x in out.stdout.strip().split(","))
    assert checked > 2_000_000_000 and bad == 0
