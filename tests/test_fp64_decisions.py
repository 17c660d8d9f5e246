"""The FP64 step's shortcut decisions (newman_gb300/csrc/pixel_fp64.cuh) --
the bailout and rebase tests decided by exponents or by FP32 estimates, Y left
unformed where both are decided, the double loop's skipped bailout sum --
against the tests they stand for, in exact agreement, on the host build of the
same header (tests/native/fp64_decisions.cpp).  CPU only."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


@pytest.fixture(scope="module")
def decisions(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("fp64") / "fp64_decisions")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "newman_gb300", "csrc"), "-I", CUDA_INC,
                    os.path.join(HERE, "native", "fp64_decisions.cpp"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("seed", [7, 2026])
def test_fp64_shortcut_decisions_match(decisions, seed):
    out = subprocess.run([decisions, "1000000", str(seed)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout[-3000:]
    assert " 0 mismatches" in out.stdout
