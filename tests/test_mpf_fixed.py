"""newman_gb300/csrc/mpf_fixed.cuh -- the fixed-precision arithmetic the
reference-exact GPU path runs -- against GMP's own mpf functions.

The reference computes in GMP mpf (gmpxx), whose operations truncate their
operands and results at limb boundaries set by the destination's precision.
tests/native/mpf_conformance.cpp drives the header's host build and
libgmp.so.10 with the same structured random operands (P = 2..19 limbs of
precision, cancelling limbs, borrow chains, exponent steps) and whole orbits
of the reference's step, and compares every result limb for limb.  CPU only.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def conformance(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("mpf") / "mpf_conformance")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "newman_gb300", "csrc"),
                    os.path.join(HERE, "native", "mpf_conformance.cpp"), "-o", exe,
                    "-l:libgmp.so.10"], check=True)
    return exe


@pytest.mark.parametrize("seed", [2026, 7])
def test_mpf_fixed_matches_gmp(conformance, seed):
    out = subprocess.run([conformance, "200000", str(seed)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-3000:]
    assert " 0 mismatches" in out.stdout
