"""The integer FP64 routines of the kernels (pg_ieee64.cuh: division, square root, addition,
subtraction, multiplication, FP32 -> FP64 conversion, the compare a > b for b >= +0) give the bits
of the IEEE operations: host build of the same routines (tests/native/ieee64_check.cpp) against the
host's IEEE operations, with the FP32 estimates exact and with them scaled by
1 +- 2^-20, at least four times the error of the GPU's estimates, to check the correction margins.
CPU only."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "perigrain_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
@pytest.mark.parametrize("scale,cases", [("1.0f", 1000000), ("1.000000953674316f", 200000),
                                         ("0.999999046325684f", 200000)])
def test_integer_div_sqrt_match_ieee(scale, cases):
    d = tempfile.mkdtemp(prefix="ieee64_")
    exe = os.path.join(d, "ieee64_check")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", f"-DPG_IEEE64_EST_SCALE={scale}", "-I", CSRC,
                    os.path.join(HERE, "native", "ieee64_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, str(cases), "97"], capture_output=True, text=True, timeout=300).stdout
    assert out.strip().endswith("bad 0"), out
