"""The smoothers' divisions by the diagonal count without a divide
instruction (Markstein's FMA correction): div6_rn (flub_gb300/csrc/smooth8.cuh)
must equal IEEE single-precision a / 6 for every float32 in the range the
kernels send through it, and ddiv_small_rn (flub_gb300/csrc/tail.cuh, the
FP64 bottom) IEEE double a / d for d = 1..6 on 2^28 random doubles per d.
Compiled and run on the host (gcc, OpenMP), seconds on 8 cores."""
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


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_fp64_small_division_matches_ieee_on_random_doubles():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "ddiv_check")
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-o", exe,
                        os.path.join(HERE, "native", "ddiv_check.c"), "-lm"], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, timeout=1200)
    assert out.returncode == 0, out.stdout + out.stderr
    checked, bad = (int(x.split()[-1]) for x in out.stdout.strip().split(","))
    assert checked == 6 << 28 and bad == 0
