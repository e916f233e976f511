"""The integer-pipe binary64 routines (blazingsql_gb300/csrc/fp64emu.cuh) give
the same bits as IEEE-754 hardware arithmetic: checked here on the host CPU
(the header compiles for the host) over millions of mixed random operands,
with the reciprocal seed deliberately perturbed by up to 2 ulp (worse than the
GPU's rcp.approx).  The GPU parity tests then cover the device build."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker():
    out = os.path.join(tempfile.mkdtemp(), "fp64emu_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-DGXE_TEST_PERTURB_RCP",
                    "-I", os.path.join(ROOT, "blazingsql_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "fp64emu_check.cpp"), "-o", out], check=True)
    return out


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_fp64_emulation_bit_exact(checker, seed):
    r = subprocess.run([checker, "1000000", str(seed)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "mismatches=0" in r.stdout
